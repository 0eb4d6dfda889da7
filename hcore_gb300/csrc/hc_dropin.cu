// hcore-gb300 — the reference's C entry points (include/hcore_d.h,
// include/hcore_s.h) on the GPU, plus the batched dense-C API.
//
// Each drop-in call validates its arguments exactly where the reference
// would exit(-1), stages pageable host buffers into a per-thread device
// arena (device and pinned pointers are used in place), runs the same
// kernels as the batched path with a batch of one on the calling thread's own
// stream, copies the results back and updates the caller's flop counter with
// the reference's model.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <thread>
#include <vector>

#include "hc_host.h"
#include "hc_zinternal.h"
#include "hcore_d.h"
#include "hcore_s.h"
#include "hcore_z.h"

// ---- the reference's globals -------------------------------------------------
extern "C" {
int use_trmm = 0;           // hcore_dgemm.c:37 (no effect: T = R_A R_B^T either way)
int gemm_print_index = 0;   // hcore_dgemm.c:41
int gemm_print_mat = 0;     // hcore_dgemm.c:42
int hc_nelm_limit = 512;    // hcore_dgemm.c:43
int sgemm_use_trmm = 0;     // hcore_sgemm.c:37
int sgemm_print_index = 0;  // hcore_sgemm.c:41
int sgemm_print_mat = 0;    // hcore_sgemm.c:42
int shc_nelm_limit = 512;   // hcore_sgemm.c:43
int syrk_print_index = 0;   // hcore_dsyrk.c:21
int gemmcd_print_index = 0; // hcore_dgemmcd.c:24
int gemmcd_print_mat = 0;   // hcore_dgemmcd.c:25
int gemmcd_use_scratch = 0; // hcore_dgemmcd.c:26
int gemmbdcd_print_index = 0;  // hcore_dgemmbdcd.c:25
int gemmbdcd_print_mat = 0;    // hcore_dgemmbdcd.c:26
// defined by the caller, as in the reference (hcore_dgemm.c:38); weak so that
// a caller without it still links and reads 0
extern int use_scratch __attribute__((weak));
}

namespace hc {

static int scratch_mode() { return &use_scratch ? use_scratch : 0; }

void fatal(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
    fflush(stderr);
    exit(-1);
}

ThreadCtx::~ThreadCtx() {
    // the runtime may already be shut down at thread/process exit: ignore errors
    if (dev) cudaFree(dev);
    if (pin) cudaFreeHost(pin);
    if (stream) cudaStreamDestroy(stream);
}

cudaError_t ThreadCtx::init() {
    if (stream) return cudaSuccess;
    return cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
}

void *ThreadCtx::dev_ensure(size_t bytes) {
    if (bytes <= dev_bytes) return dev;
    if (dev) {
        cudaStreamSynchronize(stream);
        cudaFree(dev);
    }
    dev = nullptr;
    dev_bytes = 0;
    size_t want = std::max(bytes, (size_t)1 << 20);
    if (cudaMalloc(&dev, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    dev_bytes = want;
    return dev;
}

void *ThreadCtx::pin_ensure(size_t bytes) {
    if (bytes <= pin_bytes) return pin;
    if (pin) {
        cudaStreamSynchronize(stream);
        cudaFreeHost(pin);
    }
    pin = nullptr;
    pin_bytes = 0;
    size_t want = std::max(bytes, (size_t)1 << 16);
    if (cudaMallocHost(&pin, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    pin_bytes = want;
    return pin;
}

ThreadCtx &thread_ctx() {
    static thread_local ThreadCtx ctx;
    if (ctx.init() != cudaSuccess) fatal("hcore-gb300: cannot create a CUDA stream\n");
    return ctx;
}

unsigned long flop_counts(char op, unsigned long a, unsigned long b, unsigned long c,
                          unsigned long d) {
    unsigned long res = 0;
    if (op == 'q') {  // geqrf, m >= n; single-precision division as in flop_counts.c:7
        const unsigned long m = a, n = b;
        res = 2 * m * n * n - (unsigned long)((float)(2 * n * n * n) / 3.0f) + 2 * m * n +
              (unsigned long)((float)(17 * n) / 3.0f);
    } else if (op == 'm') {
        res = a * b * c * 2;
    } else if (op == 's') {
        res = 22 * a * a * a;
    } else if (op == 'o') {
        const unsigned long m = a, n = b, k = c;
        if (d == 1) res = 4 * n * m * k - 2 * n * k * k + 3 * n * k;
        else if (d == 2) res = 4 * n * m * k - 2 * m * k * k + 2 * m * k + n * k - k * k / 2 + k / 2;
    } else if (op == 'c') {  // potrf: integer n^3/3 and n/6, n^2/2 in double (flop_counts.c:11-14)
        const unsigned long n = a;
        res = (unsigned long)(n * n * n / 3 - n * n / 2.0 + n / 6);
    } else if (op == 't') {  // trsm: side 1 (left) n m^2, side 2 (right) m n^2 (flop_counts.c:16-26)
        const unsigned long m = a, n = b;
        if (c == 1) res = n * m * m;
        else if (c == 2) res = m * n * n;
    }
    return res;
}

// flops of phase 1 (QR, factor products, SVD, scaling) of one update
static unsigned long phase1_flops(int M, int a, int b, int c, int r, bool dense_b) {
    const unsigned long k = (unsigned long)(a + c);
    unsigned long f = flop_counts('q', M, k, 0, 0);
    if (dense_b) f += flop_counts('m', M, a, M, 0);
    else f += flop_counts('m', a, b, M, 0) + flop_counts('m', M, a, b, 0);
    f += flop_counts('q', M, k, 0, 0) + flop_counts('s', k, 0, 0, 0) + (unsigned long)r * k;
    return f;
}
static unsigned long phase2_flops(int M, int k, int r) {
    return flop_counts('o', M, r, k, 1) + flop_counts('o', r, M, k, 2);
}
unsigned long update_flops(int M, int a, int b, int c, int r, bool dense_b) {
    return phase1_flops(M, a, b, c, r, dense_b) + phase2_flops(M, a + c, r);
}

static size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }
// pinned staging of a single call: descriptor at 0, rank/status at kPinRankOff
constexpr size_t kPinRankOff = 512, kPinBytes = 1024;
static_assert(sizeof(Desc) <= kPinRankOff, "descriptor larger than its pinned slot");

// ---- one update through the batched kernels --------------------------------
template <typename T>
struct Single {
    ThreadCtx &tc;
    hcore_lr_task t;
    Desc d{};
    WsLayout L{};
    int k = 0;
    char *arena = nullptr;
    T *ws = nullptr;
    Desc *d_desc = nullptr;
    int *d_rs = nullptr;  // rank, status
    T *stCU = nullptr, *stCV = nullptr;
    bool out_staged = false;

    explicit Single(const hcore_lr_task &task) : tc(thread_ctx()), t(task) {}

    // copy a host (ld x ncol) block to a packed device block with ld = rows
    void h2d(T *dst, const void *src, int rows, int ncol, int ld) {
        if (ncol <= 0) return;
        cudaMemcpy2DAsync(dst, rows * sizeof(T), src, (size_t)ld * sizeof(T), rows * sizeof(T),
                          ncol, cudaMemcpyHostToDevice, tc.stream);
    }

    // Validate, stage and upload; returns the task status (0 = runnable) or
    // -1 on a CUDA failure.  `ws_from_host` leaves the workspace for the
    // caller to fill (split API, second half).
    int prepare(unsigned flags) {
        const int st = fill_desc(t, flags, false, d, k);
        if (st) return st;
        const int M = t.M, a = t.a, b = t.b, c = t.c;
        L = ws_layout(d);
        const bool dense_b = t.Bdense != nullptr;
        bool dev_in = true;
        for (const void *p : {a ? t.AU : nullptr, a ? t.AV : nullptr,
                              dense_b ? t.Bdense : (b ? t.BU : nullptr),
                              dense_b ? nullptr : (b ? t.BV : nullptr), c ? t.CU : nullptr,
                              c ? t.CV : nullptr})
            if (p && !is_device_memory(p)) dev_in = false;
        const bool dev_out = is_device_memory(t.CUo) && is_device_memory(t.CVo);
        size_t in_elems = dev_in ? 0
                                 : (size_t)M * (2 * a + 2 * c) +
                                       (dense_b ? (size_t)M * M : (size_t)2 * M * b);
        size_t out_elems = dev_out ? 0 : (size_t)2 * M * k;
        const size_t b_in = al256(in_elems * sizeof(T)), b_out = al256(out_elems * sizeof(T));
        const size_t b_ws = al256((size_t)L.total * sizeof(T));
        const size_t total = b_in + b_out + b_ws + al256(sizeof(Desc)) + 256;
        arena = (char *)tc.dev_ensure(total);
        Desc *pin = (Desc *)tc.pin_ensure(kPinBytes);
        if (!arena || !pin) return -1;
        T *in = (T *)arena;
        stCU = (T *)(arena + b_in);
        stCV = stCU + (size_t)M * k;
        ws = (T *)(arena + b_in + b_out);
        d_desc = (Desc *)(arena + b_in + b_out + b_ws);
        d_rs = (int *)((char *)d_desc + al256(sizeof(Desc)));
        if (!dev_in) {
            T *p = in;
            if (a) {
                h2d(p, t.AU, M, a, t.lda); d.AU = p; p += (size_t)M * a;
                h2d(p, t.AV, M, a, t.lda); d.AV = p; p += (size_t)M * a;
                d.lda = M;
            }
            if (dense_b) {
                if (a) { h2d(p, t.Bdense, M, M, t.ldb); d.Bd = p; p += (size_t)M * M; d.ldb = M; }
            } else if (b) {
                h2d(p, t.BU, M, b, t.ldb); d.BU = p; p += (size_t)M * b;
                h2d(p, t.BV, M, b, t.ldb); d.BV = p; p += (size_t)M * b;
                d.ldb = M;
            }
            if (c) {
                h2d(p, t.CU, M, c, t.ldc); d.CU = p; p += (size_t)M * c;
                h2d(p, t.CV, M, c, t.ldc); d.CV = p; p += (size_t)M * c;
                d.ldc = M;
            }
        }
        out_staged = !dev_out;
        if (out_staged) {
            d.CUo = stCU;
            d.CVo = stCV;
            d.ldco = M;
        }
        d.ws = 0;
        d.idx = 0;
        d.status0 = 0;
        *pin = d;
        cudaMemcpyAsync(d_desc, pin, sizeof(Desc), cudaMemcpyHostToDevice, tc.stream);
        return cudaGetLastError() == cudaSuccess ? 0 : -1;
    }

    // run phases, fetch rank and status
    int run(unsigned phases, int *rank, int *status) {
        LaunchShape shape;
        shape.maxM = t.M;
        shape.maxK = k;
        shape.nbuckets = 1;
        shape.buckets[0] = Bucket{0, 1, k};
        // one update alone: its latency is the call's, so the Jacobi takes
        // four lanes per column pair (spread over four sub-partitions) and
        // the QR CTAs eight warps
        shape.svd_lanes[0] = shape.svd_lanes[1] = shape.svd_lanes[2] = 4;
        shape.qr_warps = 8;
        cudaError_t e = configure_recompress<T>(k, &shape.svd_smem_kmax, &shape.svd_half_kmax);
        if (e == cudaSuccess)
            e = launch_recompress<T>(d_desc, 1, ws, d_rs, d_rs + 1, nullptr, shape, tc.stream,
                                     phases);
        int *pin = (int *)((char *)tc.pin_ensure(kPinBytes) + kPinRankOff);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(pin, d_rs, 2 * sizeof(int), cudaMemcpyDeviceToHost, tc.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(tc.stream);
        if (e != cudaSuccess) return -1;
        *rank = pin[0];
        *status = pin[1];
        return 0;
    }

    // copy r result columns back to the caller's CU/CV when they were staged
    int fetch(int r) {
        if (out_staged && r > 0) {
            cudaMemcpy2DAsync(t.CUo, (size_t)t.ldco * sizeof(T), stCU, t.M * sizeof(T),
                              t.M * sizeof(T), r, cudaMemcpyDeviceToHost, tc.stream);
            cudaMemcpy2DAsync(t.CVo, (size_t)t.ldco * sizeof(T), stCV, t.M * sizeof(T),
                              t.M * sizeof(T), r, cudaMemcpyDeviceToHost, tc.stream);
        }
        return cudaStreamSynchronize(tc.stream) == cudaSuccess ? 0 : -1;
    }
};

static void cuda_fatal(const char *where) {
    fatal("%s: CUDA error: %s\n", where, cudaGetErrorString(cudaGetLastError()));
}

// HCORE_dgemm / HCORE_sgemm / HCORE_dgemm_fast share this body.
template <typename T>
static void lr_update(const char *fn, int M, T alpha, T *AU, T *AV, T *Ark, int LDA, T *BU,
                      T *BV, T *Brk, int LDB, T beta, T *CU, T *CV, T *Crk, int LDC, int rk,
                      int maxrk, T acc, flop_counter *flops, bool fast) {
    const int a = (int)Ark[0], b = (int)Brk[0], c = (int)Crk[0];
    if (!fast && (a == 0 || b == 0 || c == 0))  // hcore_dgemm.c:743-746
        fatal("%s: _Ark=%d _Brk=%d _Crk=%d. These rank values should not be zero.\n", fn, a, b, c);
    if (!fast && a + c > 2 * maxrk)  // __qra, hcore_dgemm.c:91-95
        fatal("%s: Sum of ranks (%d) is too big! _Ark:%d _Crk:%d maxrank:%d (x2: %d)\n", fn,
              a + c, a, c, maxrk, 2 * maxrk);
    if (!fast && maxrk < a + c)  // ld_newV = maxrk, hcore_dgemm.c:924-927
        fatal("%s: Increase maxrank. %d is not enough ld_newV:%d CU_ncols:%d\n", fn, maxrk,
              maxrk, a + c);
    hcore_lr_task t{};
    t.M = M; t.a = a; t.b = b; t.c = c; t.rk = rk; t.maxrk = maxrk; t.ld_newv = maxrk;
    t.alpha = alpha; t.beta = beta; t.acc = acc;
    t.AU = AU; t.AV = AV; t.lda = LDA; t.BU = BU; t.BV = BV; t.ldb = LDB;
    t.CU = CU; t.CV = CV; t.ldc = LDC; t.CUo = CU; t.CVo = CV; t.ldco = LDC;
    Single<T> s(t);
    int st = s.prepare(fast ? HCORE_GPU_FAST_RULES : 0);
    if (st < 0) cuda_fatal(fn);
    if (st) fatal("%s: invalid update (status %d): M=%d ranks %d,%d,%d maxrk=%d\n", fn, st, M, a,
                  b, c, maxrk);
    int r = 0;
    if (s.run(kPhaseAll, &r, &st)) cuda_fatal(fn);
    if (st == HCORE_GPU_S_RANK_MAX)  // hcore_dgemm.c:465-468
        fatal("%s: Rank after truncation is too big! finalrank:%d maxrank:%d\n", fn, r, maxrk);
    if (st) fatal("%s: recompression failed (status %d)\n", fn, st);
    if (s.fetch(r)) cuda_fatal(fn);
    Crk[0] = (T)r;
    if (flops) flops->update += update_flops(M, a, b, c, r, false);
}

// ---- split API (hcore_dgemm.c:1022-1699) -----------------------------------
// The first half runs stack/QR/SVD on the GPU and returns the intermediate
// state in host buffers laid out as the reference leaves them: _CU/_CV (the
// clones) hold the two QR factorizations (M x CU_ncols, ld M), qrtauA/B the
// reflector scalars, newU (ld nb) the left singular vectors and newV
// (ld 2*maxrk) the rows S V^T.  The second half uploads that state and
// rebuilds the factors into _CU_save/_CV_save.
template <typename T>
static void split_first_half(const char *fn, int M, T alpha, T *AU, T *AV, int *Ark, int LDA,
                             T *BU, T *BV, int *Brk, T *Bdense, int LDB, T beta, T *CU, T *CV,
                             int *Crk, int LDC, int rk, int storage_maxrank, int maxrk, T acc,
                             T *work, flop_counter *flops, T **_p_work_new, T **_p__CU,
                             T **_p__CV, int *_p_CU_ncols, int *_p_new_UVrk, T **_p_newU,
                             int *_p_ld_newU, T **_p_qrtauA, int *_p_CV_ncols, T **_p_newV,
                             int *_p_ld_newV, T **_p_qrtauB, int *_p_use_CUV_clone,
                             T **_p_CUclone, int *_p_ld_CUclone, T **_p__CU_save, T **_p_CVclone,
                             int *_p_ld_CVclone, T **_p__CV_save) {
    const int a = Ark[0], b = Brk ? Brk[0] : 0, c = Crk[0];
    const bool dense_b = Bdense != nullptr;
    if (dense_b && (a == 0 || c == 0))  // hcore_dgemm.c:1077-1080
        fatal("%s: _Ark=%d _Crk=%d. These rank values should not be zero.\n", fn, a, c);
    if (a + c > 2 * maxrk)
        fatal("%s: Sum of ranks (%d) is too big! _Ark:%d _Crk:%d maxrank:%d (x2: %d)\n", fn,
              a + c, a, c, maxrk, 2 * maxrk);
    if (a + c == 0)  // hcore_dgemm.c:1462-1465
        fatal("%s: CU_ncols=0 CV_ncols=0. These values should not be zero.\n", fn);
    const int k = a + c;
    const int ld_newU = M, ld_newV = 2 * maxrk;  // :1479-1480
    if (ld_newV < k)
        fatal("%s: Increase computation maxrank. %d is not enough ld_newV:%d CU_ncols:%d\n", fn,
              maxrk, ld_newV, k);
    hcore_lr_task t{};
    t.M = M; t.a = a; t.b = b; t.c = c; t.rk = rk; t.maxrk = maxrk; t.ld_newv = ld_newV;
    t.alpha = alpha; t.beta = beta; t.acc = acc;
    t.AU = AU; t.AV = AV; t.lda = LDA; t.BU = BU; t.BV = BV; t.ldb = LDB; t.Bdense = Bdense;
    t.CU = CU; t.CV = CV; t.ldc = LDC; t.CUo = CU; t.CVo = CV; t.ldco = LDC;
    Single<T> s(t);
    int st = s.prepare(0);
    if (st < 0) cuda_fatal(fn);
    if (st) fatal("%s: invalid update (status %d)\n", fn, st);
    int r = 0;
    if (s.run(kPhaseStack | kPhaseQR | kPhaseSVD, &r, &st)) cuda_fatal(fn);
    if (st == HCORE_GPU_S_RANK_MAX)
        fatal("%s: Rank after truncation is too big! finalrank:%d maxrank:%d\n", fn, r, maxrk);
    if (st) fatal("%s: recompression failed (status %d)\n", fn, st);

    // host buffers in the reference's layout (:1395-1450, :1474-1495)
    T *CUclone, *CVclone, *tauA, *tauB, *newU, *newV;
    const size_t clone_n = (size_t)M * 2 * maxrk;
    if (scratch_mode()) {
        CUclone = work; work += clone_n;
        CVclone = work; work += clone_n;
        tauA = work;
        tauB = work + M;
        newU = work + 2 * M + (size_t)maxrk * maxrk;
        newV = newU + (size_t)ld_newU * 2 * maxrk;
    } else {
        CUclone = (T *)malloc(clone_n * sizeof(T));
        CVclone = (T *)malloc(clone_n * sizeof(T));
        tauA = (T *)malloc((size_t)M * sizeof(T));
        tauB = (T *)malloc((size_t)M * sizeof(T));
        newU = (T *)malloc((size_t)ld_newU * 2 * maxrk * sizeof(T));
        newV = (T *)malloc((size_t)M * ld_newV * sizeof(T));
    }
    cudaStream_t st_ = s.tc.stream;
    const WsLayout &L = s.L;
    cudaMemcpyAsync(CUclone, s.ws + L.UA, (size_t)M * k * sizeof(T), cudaMemcpyDeviceToHost, st_);
    cudaMemcpyAsync(CVclone, s.ws + L.VB, (size_t)M * k * sizeof(T), cudaMemcpyDeviceToHost, st_);
    cudaMemcpyAsync(tauA, s.ws + L.tauA, k * sizeof(T), cudaMemcpyDeviceToHost, st_);
    cudaMemcpyAsync(tauB, s.ws + L.tauB, k * sizeof(T), cudaMemcpyDeviceToHost, st_);
    std::vector<T> Uo((size_t)k * (r > 0 ? r : 1)), Vo((size_t)k * (r > 0 ? r : 1));
    if (r > 0) {
        cudaMemcpyAsync(Uo.data(), s.ws + L.Uo, (size_t)k * r * sizeof(T), cudaMemcpyDeviceToHost, st_);
        cudaMemcpyAsync(Vo.data(), s.ws + L.Vo, (size_t)k * r * sizeof(T), cudaMemcpyDeviceToHost, st_);
    }
    if (cudaStreamSynchronize(st_) != cudaSuccess) cuda_fatal(fn);
    for (int j = 0; j < r; ++j)
        for (int i = 0; i < k; ++i) {
            newU[(size_t)j * ld_newU + i] = Uo[(size_t)j * k + i];  // U(:, j)
            newV[(size_t)i * ld_newV + j] = Vo[(size_t)j * k + i];  // (S V^T)(j, i)
        }
    if (flops) flops->update += phase1_flops(M, a, b, c, r, dense_b);
    *_p_work_new = work;
    *_p__CU = CUclone;
    *_p__CV = CVclone;
    *_p_CU_ncols = k;
    *_p_new_UVrk = r;
    *_p_newU = newU;
    *_p_ld_newU = ld_newU;
    *_p_qrtauA = tauA;
    *_p_CV_ncols = k;
    *_p_newV = newV;
    *_p_ld_newV = ld_newV;
    *_p_qrtauB = tauB;
    *_p_use_CUV_clone = 1;
    *_p_CUclone = CUclone;
    *_p_ld_CUclone = M;
    *_p__CU_save = CU;
    *_p_CVclone = CVclone;
    *_p_ld_CVclone = M;
    *_p__CV_save = CV;
}

template <typename T>
static void split_second_half(const char *fn, int M, int *Crk, int LDC, int storage_maxrank,
                              flop_counter *flops, T *_CU, T *_CV, int CU_ncols, int new_UVrk,
                              T *newU, int ld_newU, T *qrtauA, int CV_ncols, T *newV,
                              int ld_newV, T *qrtauB, int use_CUV_clone, T *CUclone, T *_CU_save,
                              T *CVclone, T *_CV_save) {
    if (new_UVrk > storage_maxrank)  // hcore_dgemm.c:1648-1651
        fatal("%s: Increase storage maxrank %d. Observed rank for U and V is %d\n", fn,
              storage_maxrank, new_UVrk);
    const int k = CU_ncols, r = new_UVrk;
    if (CV_ncols != k || k > M) fatal("%s: inconsistent factor widths %d/%d\n", fn, CU_ncols, CV_ncols);
    // a task whose first three phases are replaced by the uploaded state
    hcore_lr_task t{};
    t.M = M; t.a = k; t.b = 0; t.c = 0; t.rk = r > 0 ? r : 1; t.maxrk = k; t.ld_newv = k;
    t.alpha = 1; t.beta = 1; t.acc = 0;
    t.AU = _CU; t.AV = _CU; t.lda = M;
    t.CUo = _CU_save; t.CVo = _CV_save; t.ldco = LDC;
    Single<T> s(t);
    int st = s.prepare(0);
    if (st < 0) cuda_fatal(fn);
    if (st) fatal("%s: invalid state (status %d)\n", fn, st);
    if (r > 0) {
        cudaStream_t st_ = s.tc.stream;
        const WsLayout &L = s.L;
        std::vector<T> Uo((size_t)k * r), Vo((size_t)k * r);
        for (int j = 0; j < r; ++j)
            for (int i = 0; i < k; ++i) {
                Uo[(size_t)j * k + i] = newU[(size_t)j * ld_newU + i];
                Vo[(size_t)j * k + i] = newV[(size_t)i * ld_newV + j];
            }
        cudaMemcpyAsync(s.ws + L.UA, _CU, (size_t)M * k * sizeof(T), cudaMemcpyHostToDevice, st_);
        cudaMemcpyAsync(s.ws + L.VB, _CV, (size_t)M * k * sizeof(T), cudaMemcpyHostToDevice, st_);
        cudaMemcpyAsync(s.ws + L.tauA, qrtauA, k * sizeof(T), cudaMemcpyHostToDevice, st_);
        cudaMemcpyAsync(s.ws + L.tauB, qrtauB, k * sizeof(T), cudaMemcpyHostToDevice, st_);
        cudaMemcpyAsync(s.ws + L.Uo, Uo.data(), (size_t)k * r * sizeof(T), cudaMemcpyHostToDevice, st_);
        cudaMemcpyAsync(s.ws + L.Vo, Vo.data(), (size_t)k * r * sizeof(T), cudaMemcpyHostToDevice, st_);
        const int rs[2] = {r, 0};
        // the descriptor upload still reads the start of the pinned buffer;
        // the rank slot lives past it
        int *pin = (int *)((char *)s.tc.pin_ensure(kPinBytes) + kPinRankOff + 64);
        pin[0] = rs[0];
        pin[1] = rs[1];
        cudaMemcpyAsync(s.d_rs, pin, 2 * sizeof(int), cudaMemcpyHostToDevice, st_);
        int rr = 0, sst = 0;
        if (s.run(kPhaseApply, &rr, &sst)) cuda_fatal(fn);
        if (s.fetch(r)) cuda_fatal(fn);
    }
    if (use_CUV_clone == 1 && !scratch_mode()) {
        free(CUclone);
        free(CVclone);
    }
    if (!scratch_mode()) {
        free(qrtauA);
        free(qrtauB);
        free(newU);
        free(newV);
    }
    Crk[0] = r;
    if (flops) flops->update += phase2_flops(M, k, r);
}

// ---- dense updates -----------------------------------------------------------
struct DenseRun {
    ThreadCtx &tc;
    DenseRun() : tc(thread_ctx()) {}
};

// Host-side preparation of a list of dense tasks (device-accessible
// pointers): group by output tile (list order kept inside each group), the
// rank-K' form of every task and the workspace layout.
struct DensePrep {
    int n = 0, maxDim = 1, maxN3 = 0, maxA3 = 0;
    std::vector<DenseWork> work;
    std::vector<int> gstart, gtasks, bdcd;  // bdcd: the gemmbdcd tasks
    long long ws = 0;  // doubles
    size_t b_tasks = 0, b_work = 0, b_gs = 0, b_gt = 0, b_bd = 0, b_ws = 0;
    size_t bytes() const { return b_tasks + b_work + b_gs + b_gt + b_bd + b_ws; }
    size_t ws_offset() const { return b_tasks + b_work + b_gs + b_gt + b_bd; }
    int ngroups() const { return (int)gstart.size() - 1; }

    static bool valid(const hcore_dense_task &t) {
        const int N = t.N ? t.N : t.M;
        if (t.M < 1 || N < 1 || t.a < 0 || t.b < 0 || !t.CD || t.ldcd < t.M) return false;
        switch (t.kind) {
        case 0:
        case 1:
            return N == t.M;
        case 2:
            return t.a == 0 || (t.Au && t.Bv && t.lda >= t.M && t.ldb >= N);
        case 3: {
            const int K = t.kdim ? t.kdim : t.M;
            return K >= 1 && (t.a == 0 || (t.Au && t.Av && t.Bd && t.lda >= std::max(t.M, K) &&
                                           t.ldb >= K));
        }
        default:
            return false;
        }
    }

    int build(int n_, const hcore_dense_task *tasks) {
        n = n_;
        std::map<const double *, int> gid;
        std::vector<std::vector<int>> groups;
        work.assign(n, DenseWork{});
        bdcd.clear();
        ws = 0;
        for (int i = 0; i < n; ++i) {
            const hcore_dense_task &t = tasks[i];
            if (!valid(t)) {
                set_error("dense tasks: invalid task %d", i);
                return HCORE_GPU_EINVAL;
            }
            const int N = t.N ? t.N : t.M;
            auto it = gid.find(t.CD);
            if (it == gid.end()) {
                gid[t.CD] = (int)groups.size();
                groups.push_back({i});
            } else {
                const hcore_dense_task &t0 = tasks[groups[it->second][0]];
                if (t0.M != t.M || (t0.N ? t0.N : t0.M) != N) {
                    set_error("dense tasks: tasks on one tile disagree on its shape");
                    return HCORE_GPU_EINVAL;
                }
                groups[it->second].push_back(i);
            }
            maxDim = std::max(maxDim, std::max(t.M, N));
            DenseWork &w = work[i];
            w.ws = ws;
            w.beta = 1.0;
            if (t.kind <= 1) {
                const long long sq = t.kind == 0 ? (long long)t.a * t.a : (long long)t.a * t.b;
                const int kk = t.kind == 0 ? t.a : std::min(t.a, t.b);
                ws += ((sq + (long long)t.M * kk + 31) / 32) * 32;
                w.syrk = t.kind == 0;
                w.kk = kk;
                w.coef = t.kind == 0 ? t.alpha : -1.0;
            } else if (t.kind == 2) {  // alpha = 1, beta = 0 (hcore_duncompress.c:73-79)
                w.kk = t.a;
                w.coef = 1.0;
                w.beta = 0.0;
            } else {
                w.kk = t.a;
                w.coef = t.alpha;
                w.beta = t.beta;
                if (t.a > 0) {
                    ws += (((long long)N * t.a + 31) / 32) * 32;
                    bdcd.push_back(i);
                    maxN3 = std::max(maxN3, N);
                    maxA3 = std::max(maxA3, t.a);
                }
            }
        }
        gstart.assign(groups.size() + 1, 0);
        gtasks.clear();
        for (size_t g = 0; g < groups.size(); ++g) {
            gstart[g + 1] = gstart[g] + (int)groups[g].size();
            for (int i : groups[g]) gtasks.push_back(i);
        }
        b_tasks = al256(n * sizeof(hcore_dense_task));
        b_work = al256(n * sizeof(DenseWork));
        b_gs = al256(gstart.size() * sizeof(int));
        b_gt = al256(gtasks.size() * sizeof(int));
        b_bd = al256(std::max<size_t>(bdcd.size(), 1) * sizeof(int));
        b_ws = al256((size_t)ws * sizeof(double));
        return HCORE_GPU_OK;
    }

    // point each task's P/Q at its inputs or at its computed factor in the
    // workspace that starts at d_ws
    void bind(const hcore_dense_task *tasks, const double *d_ws) {
        for (int i = 0; i < n; ++i) {
            const hcore_dense_task &t = tasks[i];
            DenseWork &w = work[i];
            const int N = t.N ? t.N : t.M;
            if (t.kind == 2) {
                w.P = t.Au; w.ldp = t.lda; w.Q = t.Bv; w.ldq = t.ldb;
                continue;
            }
            if (t.kind == 3) {
                w.P = t.Au; w.ldp = t.lda; w.Q = d_ws + w.ws; w.ldq = N;
                continue;
            }
            const long long sq = t.kind == 0 ? (long long)t.a * t.a : (long long)t.a * t.b;
            const double *computed = d_ws + w.ws + sq;
            if (t.kind == 0) {
                w.P = computed; w.ldp = t.M; w.Q = t.Au; w.ldq = t.lda;
            } else if (t.a > t.b) {
                w.P = computed; w.ldp = t.M; w.Q = t.Bu; w.ldq = t.M;
            } else {
                w.P = t.Au; w.ldp = t.M; w.Q = computed; w.ldq = t.M;
            }
        }
    }

    // copy tasks, work, groups and the gemmbdcd list into `host` (pinned or
    // not) laid out as the device arena's first ws_offset() bytes
    void pack(char *host, const hcore_dense_task *tasks) const {
        memcpy(host, tasks, n * sizeof(hcore_dense_task));
        memcpy(host + b_tasks, work.data(), n * sizeof(DenseWork));
        memcpy(host + b_tasks + b_work, gstart.data(), gstart.size() * sizeof(int));
        memcpy(host + b_tasks + b_work + b_gs, gtasks.data(), gtasks.size() * sizeof(int));
        if (!bdcd.empty())
            memcpy(host + b_tasks + b_work + b_gs + b_gt, bdcd.data(), bdcd.size() * sizeof(int));
    }

    cudaError_t launch(char *arena, cudaStream_t s) const {
        const hcore_dense_task *d_tasks = (const hcore_dense_task *)arena;
        const DenseWork *d_work = (const DenseWork *)(arena + b_tasks);
        double *d_ws = (double *)(arena + ws_offset());
        cudaError_t e = launch_dense_prep(d_tasks, d_work, n, d_ws, s);
        if (e == cudaSuccess && !bdcd.empty())
            e = launch_bdcd_prep(d_tasks, d_work, (const int *)(arena + b_tasks + b_work + b_gs + b_gt),
                                 (int)bdcd.size(), maxN3, maxA3, d_ws, s);
        if (e == cudaSuccess)
            e = launch_dense_tiles(d_tasks, d_work, (const int *)(arena + b_tasks + b_work),
                                   (const int *)(arena + b_tasks + b_work + b_gs), ngroups(),
                                   maxDim, s);
        return e;
    }
};

// Run a list of dense tasks (device-accessible pointers) on stream s, in the
// calling thread's arena.
static int run_dense(int n, const hcore_dense_task *tasks, cudaStream_t s, bool sync) {
    if (n <= 0) return HCORE_GPU_OK;
    DensePrep dp;
    int rc = dp.build(n, tasks);
    if (rc) return rc;
    ThreadCtx &tc = thread_ctx();
    char *arena = (char *)tc.dev_ensure(dp.bytes());
    char *pin = (char *)tc.pin_ensure(dp.ws_offset());
    if (!arena || !pin) {
        set_error("hcore_gpu_dense_batched: out of memory");
        return HCORE_GPU_ENOMEM;
    }
    dp.bind(tasks, (const double *)(arena + dp.ws_offset()));
    // the previous call on this stream may still read the pinned buffer
    cudaStreamSynchronize(s);
    dp.pack(pin, tasks);
    cudaMemcpyAsync(arena, pin, dp.ws_offset(), cudaMemcpyHostToDevice, s);
    cudaError_t e = dp.launch(arena, s);
    if (e == cudaSuccess && sync) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_dense_batched: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    return HCORE_GPU_OK;
}

// stage one dense host block (rows x cols, ld) into dst (ld rows)
static void stage(double *dst, const double *src, int rows, int cols, int ld, cudaStream_t s) {
    if (cols > 0 && rows > 0)
        cudaMemcpy2DAsync(dst, rows * sizeof(double), src, (size_t)ld * sizeof(double),
                          rows * sizeof(double), cols, cudaMemcpyHostToDevice, s);
}

// the same into dst with leading dimension ldd >= rows
static void stage_ld(double *dst, int ldd, const double *src, int rows, int cols, int ld,
                     cudaStream_t s) {
    if (cols > 0 && rows > 0)
        cudaMemcpy2DAsync(dst, (size_t)ldd * sizeof(double), src, (size_t)ld * sizeof(double),
                          rows * sizeof(double), cols, cudaMemcpyHostToDevice, s);
}

// copy a dense device block (rows x cols, ld rows) back to the caller's host
// block (ld) and wait for it
static void unstage(double *dst, int ld, const double *src, int rows, int cols, cudaStream_t s,
                    const char *fn) {
    if (rows > 0 && cols > 0)
        cudaMemcpy2DAsync(dst, (size_t)ld * sizeof(double), src, rows * sizeof(double),
                          rows * sizeof(double), cols, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) cuda_fatal(fn);
}

// per-thread device buffer of at least n doubles for the host operands of the
// dense drop-ins (the dense runner itself uses the thread arena)
static double *stage_buffer(size_t n, const char *fn) {
    static thread_local double *buf = nullptr;
    static thread_local size_t buf_n = 0;
    if (buf_n < n) {
        if (buf) {
            cudaStreamSynchronize(thread_ctx().stream);
            cudaFree(buf);
        }
        buf = nullptr;
        buf_n = 0;
        if (cudaMalloc(&buf, std::max<size_t>(n, 1) * sizeof(double)) != cudaSuccess)
            fatal("%s: cannot allocate %zu bytes of device memory\n", fn, n * sizeof(double));
        buf_n = n;
    }
    return buf;
}

}  // namespace hc

using namespace hc;

extern "C" {

void HCORE_dgemm(HCORE_enum transA, int transB, int M, int N, double alpha, double *AU,
                 double *AV, double *Ark, int LDA, double *BU, double *BV, double *Brk, int LDB,
                 double beta, double *CU, double *CV, double *Crk, int LDC, int rk, int maxrk,
                 double acc, double *work, flop_counter *flops) {
    (void)transA; (void)transB; (void)N; (void)work;
    lr_update<double>("HCORE_dgemm", M, alpha, AU, AV, Ark, LDA, BU, BV, Brk, LDB, beta, CU, CV,
                      Crk, LDC, rk, maxrk, acc, flops, false);
}

void HCORE_sgemm(HCORE_enum transA, HCORE_enum transB, int M, int N, float alpha, float *AU,
                 float *AV, float *Ark, int LDA, float *BU, float *BV, float *Brk, int LDB,
                 float beta, float *CU, float *CV, float *Crk, int LDC, int rk, int maxrk,
                 float acc, float *work, flop_counter *flops) {
    (void)transA; (void)transB; (void)N; (void)work;
    lr_update<float>("HCORE_sgemm", M, alpha, AU, AV, Ark, LDA, BU, BV, Brk, LDB, beta, CU, CV,
                     Crk, LDC, rk, maxrk, acc, flops, false);
}

void HCORE_dgemm_fast(HCORE_enum transA, int transB, int M, int N, double alpha, double *AU,
                      double *AV, double *Ark, int LDA, double *BU, double *BV, double *Brk,
                      int LDB, double beta, double *CU, double *CV, double *Crk, int LDC, int rk,
                      int maxrk, double acc, double *work) {
    (void)transA; (void)transB; (void)N; (void)work;
    lr_update<double>("HCORE_dgemm_fast", M, alpha, AU, AV, Ark, LDA, BU, BV, Brk, LDB, beta, CU,
                      CV, Crk, LDC, rk, maxrk, acc, nullptr, true);
}

void HCORE_dgemm_qr_svd(int transA, int transB, int M, int N, double alpha, double *AU,
                        double *AV, int *Ark, int LDA, double *BU, double *BV, int *Brk, int LDB,
                        double beta, double *CU, double *CV, int *Crk, int LDC, int rk,
                        int storage_maxrank, int maxrk, double acc, double *work,
                        flop_counter *flops, double **_p_work_new, double **_p__CU,
                        double **_p__CV, int *_p_CU_ncols, int *_p_new_UVrk, double **_p_newU,
                        int *_p_ld_newU, double **_p_qrtauA, int *_p_CV_ncols, double **_p_newV,
                        int *_p_ld_newV, double **_p_qrtauB, int *_p_use_CUV_clone,
                        double **_p_CUclone, int *_p_ld_CUclone, double **_p__CU_save,
                        double **_p_CVclone, int *_p_ld_CVclone, double **_p__CV_save) {
    (void)transA; (void)transB; (void)N;
    split_first_half<double>("HCORE_dgemm_qr_svd", M, alpha, AU, AV, Ark, LDA, BU, BV, Brk,
                             nullptr, LDB, beta, CU, CV, Crk, LDC, rk, storage_maxrank, maxrk,
                             acc, work, flops, _p_work_new, _p__CU, _p__CV, _p_CU_ncols,
                             _p_new_UVrk, _p_newU, _p_ld_newU, _p_qrtauA, _p_CV_ncols, _p_newV,
                             _p_ld_newV, _p_qrtauB, _p_use_CUV_clone, _p_CUclone, _p_ld_CUclone,
                             _p__CU_save, _p_CVclone, _p_ld_CVclone, _p__CV_save);
}

void HCORE_dgemm_qr_svd_b_dense(int transA, int transB, int M, int N, double alpha, double *AU,
                                double *AV, int *Ark, int LDA, double *B, int LDB, double beta,
                                double *CU, double *CV, int *Crk, int LDC, int rk,
                                int storage_maxrank, int maxrk, double acc, double *work,
                                flop_counter *flops, double **_p_work_new, double **_p__CU,
                                double **_p__CV, int *_p_CU_ncols, int *_p_new_UVrk,
                                double **_p_newU, int *_p_ld_newU, double **_p_qrtauA,
                                int *_p_CV_ncols, double **_p_newV, int *_p_ld_newV,
                                double **_p_qrtauB, int *_p_use_CUV_clone, double **_p_CUclone,
                                int *_p_ld_CUclone, double **_p__CU_save, double **_p_CVclone,
                                int *_p_ld_CVclone, double **_p__CV_save) {
    (void)transA; (void)transB; (void)N;
    split_first_half<double>("HCORE_dgemm_qr_svd_b_dense", M, alpha, AU, AV, Ark, LDA, nullptr,
                             nullptr, nullptr, B, LDB, beta, CU, CV, Crk, LDC, rk,
                             storage_maxrank, maxrk, acc, work, flops, _p_work_new, _p__CU,
                             _p__CV, _p_CU_ncols, _p_new_UVrk, _p_newU, _p_ld_newU, _p_qrtauA,
                             _p_CV_ncols, _p_newV, _p_ld_newV, _p_qrtauB, _p_use_CUV_clone,
                             _p_CUclone, _p_ld_CUclone, _p__CU_save, _p_CVclone, _p_ld_CVclone,
                             _p__CV_save);
}

void HCORE_dgemm_ormqr(int transA, int transB, int M, int N, double alpha, double *AU,
                       double *AV, int *Ark, int LDA, double beta, double *CU, double *CV,
                       int *Crk, int LDC, int rk, int storage_maxrank, int maxrk, double acc,
                       double *work, flop_counter *flops, double *_CU, double *_CV,
                       int CU_ncols, int new_UVrk, double *newU, int ld_newU, double *qrtauA,
                       int CV_ncols, double *newV, int ld_newV, double *qrtauB,
                       int use_CUV_clone, double *CUclone, int ld_CUclone, double *_CU_save,
                       double *CVclone, int ld_CVclone, double *_CV_save) {
    (void)transA; (void)transB; (void)N; (void)alpha; (void)AU; (void)AV; (void)Ark; (void)LDA;
    (void)beta; (void)CU; (void)CV; (void)rk; (void)maxrk; (void)acc; (void)work;
    (void)ld_CUclone; (void)ld_CVclone;
    split_second_half<double>("HCORE_dgemm_ormqr", M, Crk, LDC, storage_maxrank, flops, _CU, _CV,
                              CU_ncols, new_UVrk, newU, ld_newU, qrtauA, CV_ncols, newV, ld_newV,
                              qrtauB, use_CUV_clone, CUclone, _CU_save, CVclone, _CV_save);
}

void HCORE_sgemm_qr_svd(int transA, int transB, int M, int N, float alpha, float *AU, float *AV,
                        int *Ark, int LDA, float *BU, float *BV, int *Brk, int LDB, float beta,
                        float *CU, float *CV, int *Crk, int LDC, int rk, int storage_maxrank,
                        int maxrk, float acc, float *work, flop_counter *flops,
                        float **_p_work_new, float **_p__CU, float **_p__CV, int *_p_CU_ncols,
                        int *_p_new_UVrk, float **_p_newU, int *_p_ld_newU, float **_p_qrtauA,
                        int *_p_CV_ncols, float **_p_newV, int *_p_ld_newV, float **_p_qrtauB,
                        int *_p_use_CUV_clone, float **_p_CUclone, int *_p_ld_CUclone,
                        float **_p__CU_save, float **_p_CVclone, int *_p_ld_CVclone,
                        float **_p__CV_save) {
    (void)transA; (void)transB; (void)N;
    split_first_half<float>("HCORE_sgemm_qr_svd", M, alpha, AU, AV, Ark, LDA, BU, BV, Brk,
                            nullptr, LDB, beta, CU, CV, Crk, LDC, rk, storage_maxrank, maxrk, acc,
                            work, flops, _p_work_new, _p__CU, _p__CV, _p_CU_ncols, _p_new_UVrk,
                            _p_newU, _p_ld_newU, _p_qrtauA, _p_CV_ncols, _p_newV, _p_ld_newV,
                            _p_qrtauB, _p_use_CUV_clone, _p_CUclone, _p_ld_CUclone, _p__CU_save,
                            _p_CVclone, _p_ld_CVclone, _p__CV_save);
}

void HCORE_sgemm_qr_svd_b_dense(int transA, int transB, int M, int N, float alpha, float *AU,
                                float *AV, int *Ark, int LDA, float *B, int LDB, float beta,
                                float *CU, float *CV, int *Crk, int LDC, int rk,
                                int storage_maxrank, int maxrk, float acc, float *work,
                                flop_counter *flops, float **_p_work_new, float **_p__CU,
                                float **_p__CV, int *_p_CU_ncols, int *_p_new_UVrk,
                                float **_p_newU, int *_p_ld_newU, float **_p_qrtauA,
                                int *_p_CV_ncols, float **_p_newV, int *_p_ld_newV,
                                float **_p_qrtauB, int *_p_use_CUV_clone, float **_p_CUclone,
                                int *_p_ld_CUclone, float **_p__CU_save, float **_p_CVclone,
                                int *_p_ld_CVclone, float **_p__CV_save) {
    (void)transA; (void)transB; (void)N;
    split_first_half<float>("HCORE_sgemm_qr_svd_b_dense", M, alpha, AU, AV, Ark, LDA, nullptr,
                            nullptr, nullptr, B, LDB, beta, CU, CV, Crk, LDC, rk, storage_maxrank,
                            maxrk, acc, work, flops, _p_work_new, _p__CU, _p__CV, _p_CU_ncols,
                            _p_new_UVrk, _p_newU, _p_ld_newU, _p_qrtauA, _p_CV_ncols, _p_newV,
                            _p_ld_newV, _p_qrtauB, _p_use_CUV_clone, _p_CUclone, _p_ld_CUclone,
                            _p__CU_save, _p_CVclone, _p_ld_CVclone, _p__CV_save);
}

void HCORE_sgemm_ormqr(int transA, int transB, int M, int N, float alpha, float *AU, float *AV,
                       int *Ark, int LDA, float beta, float *CU, float *CV, int *Crk, int LDC,
                       int rk, int storage_maxrank, int maxrk, float acc, float *work,
                       flop_counter *flops, float *_CU, float *_CV, int CU_ncols, int new_UVrk,
                       float *newU, int ld_newU, float *qrtauA, int CV_ncols, float *newV,
                       int ld_newV, float *qrtauB, int use_CUV_clone, float *CUclone,
                       int ld_CUclone, float *_CU_save, float *CVclone, int ld_CVclone,
                       float *_CV_save) {
    (void)transA; (void)transB; (void)N; (void)alpha; (void)AU; (void)AV; (void)Ark; (void)LDA;
    (void)beta; (void)CU; (void)CV; (void)rk; (void)maxrk; (void)acc; (void)work;
    (void)ld_CUclone; (void)ld_CVclone;
    split_second_half<float>("HCORE_sgemm_ormqr", M, Crk, LDC, storage_maxrank, flops, _CU, _CV,
                             CU_ncols, new_UVrk, newU, ld_newU, qrtauA, CV_ncols, newV, ld_newV,
                             qrtauB, use_CUV_clone, CUclone, _CU_save, CVclone, _CV_save);
}

void HCORE_dsyrk(HCORE_enum uplo, HCORE_enum trans, int M, int K, double alpha, const double *AU,
                 int LDAU, const double *AV, int LDAV, double beta, double *CD, int LDCD,
                 double *work, flop_counter *flops) {
    (void)uplo; (void)trans; (void)LDAV; (void)beta; (void)work;
    ThreadCtx &tc = thread_ctx();
    const int N = LDAU;  // hcore_dsyrk.c:57: AV has LDAU rows, every factor ld is LDAU
    hcore_dense_task t{};
    t.kind = 0; t.M = M; t.a = K; t.alpha = alpha;
    const bool dev = is_device_memory(AU) && is_device_memory(AV) && is_device_memory(CD);
    if (dev) {
        t.Au = AU; t.Av = AV; t.lda = LDAU; t.CD = CD; t.ldcd = LDCD;
    } else {
        const size_t nf = (size_t)N * K, nc = (size_t)M * M;
        double *buf = stage_buffer(2 * nf + nc, "HCORE_dsyrk");
        stage(buf, AU, N, K, LDAU, tc.stream);
        stage(buf + nf, AV, N, K, LDAU, tc.stream);
        stage(buf + 2 * nf, CD, M, M, LDCD, tc.stream);
        t.Au = buf; t.Av = buf + nf; t.lda = N; t.CD = buf + 2 * nf; t.ldcd = M;
    }
    if (run_dense(1, &t, tc.stream, true)) fatal("HCORE_dsyrk: %s\n", last_error());
    if (!dev) unstage(CD, LDCD, t.CD, M, M, tc.stream, "HCORE_dsyrk");
    if (flops)  // hcore_dsyrk.c:104-188
        flops->syrk += flop_counts('m', K, K, N, 0) + flop_counts('m', M, K, K, 0) +
                       flop_counts('m', M, M, K, 0);
}

void HCORE_dgemmcd(HCORE_enum transA, HCORE_enum transB, int M, double alpha, double *Au,
                   double *Av, int Arank, int LDA, double *Bu, double *Bv, int Brank, int LDB,
                   double beta, double *CD, int LDC, int maxrank, double *work,
                   flop_counter *flops) {
    (void)transA; (void)transB; (void)alpha; (void)LDA; (void)LDB; (void)beta; (void)LDC;
    (void)maxrank; (void)work; (void)flops;  // the reference counts no flops here
    ThreadCtx &tc = thread_ctx();
    hcore_dense_task t{};
    t.kind = 1; t.M = M; t.a = Arank; t.b = Brank; t.alpha = -1.0;
    const bool dev = is_device_memory(Au) && is_device_memory(Av) && is_device_memory(Bu) &&
                     is_device_memory(Bv) && is_device_memory(CD);
    if (dev) {
        t.Au = Au; t.Av = Av; t.Bu = Bu; t.Bv = Bv; t.lda = M; t.ldb = M; t.CD = CD; t.ldcd = M;
    } else {
        const size_t na = (size_t)M * Arank, nb = (size_t)M * Brank, nc = (size_t)M * M;
        double *buf = stage_buffer(2 * na + 2 * nb + nc, "HCORE_dgemmcd");
        // every leading dimension is M (hcore_dgemmcd.c:66-99)
        stage(buf, Au, M, Arank, M, tc.stream);
        stage(buf + na, Av, M, Arank, M, tc.stream);
        stage(buf + 2 * na, Bu, M, Brank, M, tc.stream);
        stage(buf + 2 * na + nb, Bv, M, Brank, M, tc.stream);
        stage(buf + 2 * na + 2 * nb, CD, M, M, M, tc.stream);
        t.Au = buf; t.Av = buf + na; t.Bu = buf + 2 * na; t.Bv = buf + 2 * na + nb;
        t.lda = M; t.ldb = M; t.CD = buf + 2 * na + 2 * nb; t.ldcd = M;
    }
    if (run_dense(1, &t, tc.stream, true)) fatal("HCORE_dgemmcd: %s\n", last_error());
    if (!dev) unstage(CD, M, t.CD, M, M, tc.stream, "HCORE_dgemmcd");
}

// CD = AU BV^T: M x N from two rank-Ark factors (hcore_duncompress.c:33-84).
// alpha and beta are not used (the reference passes 1 and 0 to its GEMM) and
// the two ranks must agree (its assert at :67).
void HCORE_duncompress(HCORE_enum transA, HCORE_enum transB, int M, int N, double alpha,
                       double *AU, double *Ark, int LDA, double *BV, double *Brk, int LDB,
                       double beta, double *CD, int LDC) {
    (void)transA; (void)transB; (void)alpha; (void)beta;
    const long long a = (long long)Ark[0], b = (long long)Brk[0];
    if (a != b) fatal("HCORE_duncompress: Ark (%lld) and Brk (%lld) must be equal\n", a, b);
    if (M <= 0 || N <= 0) return;
    ThreadCtx &tc = thread_ctx();
    hcore_dense_task t{};
    t.kind = 2; t.M = M; t.N = N; t.a = (int)a;
    const bool dev = is_device_memory(CD) && (a == 0 || (is_device_memory(AU) && is_device_memory(BV)));
    if (dev) {
        t.Au = AU; t.lda = LDA; t.Bv = BV; t.ldb = LDB; t.CD = CD; t.ldcd = LDC;
    } else {
        if (LDA < M || LDB < N || LDC < M)
            fatal("HCORE_duncompress: invalid leading dimension (LDA %d, LDB %d, LDC %d)\n", LDA,
                  LDB, LDC);
        const size_t na = (size_t)M * a, nb = (size_t)N * a;
        double *buf = stage_buffer(na + nb + (size_t)M * N, "HCORE_duncompress");
        stage(buf, AU, M, (int)a, LDA, tc.stream);
        stage(buf + na, BV, N, (int)a, LDB, tc.stream);
        t.Au = buf; t.lda = M; t.Bv = buf + na; t.ldb = N; t.CD = buf + na + nb; t.ldcd = M;
    }
    if (run_dense(1, &t, tc.stream, true)) fatal("HCORE_duncompress: %s\n", last_error());
    if (!dev) unstage(CD, LDC, t.CD, M, N, tc.stream, "HCORE_duncompress");
}

// CD = alpha AU (AV^T BD) + beta CD (hcore_dgemmbdcd.c:35-122).  As in the
// reference, transA == HCORE_Trans sums AV^T BD over M rows and gives CD LDA
// rows; otherwise the sum runs over LDB rows and CD has M rows.  Flops:
// the reference's two GEMM terms (:95-96, :114-115).
void HCORE_dgemmbdcd(HCORE_enum transA, HCORE_enum transB, int M, int N, double alpha,
                     double *AU, double *AV, double *Ark, int LDA, double *BD, int LDB,
                     double beta, double *CD, int LDC, double *work, flop_counter *flops) {
    (void)transB; (void)work;
    const long long a = (long long)Ark[0];
    const bool tr = transA == HCORE_Trans;
    const int rows = tr ? LDA : M, K = tr ? M : LDB;
    if (flops)
        flops->update += flop_counts('m', (unsigned long)a, N, K, 0) +
                         flop_counts('m', rows, N, (unsigned long)a, 0);
    // a = 0: the reference hands BLAS a leading dimension of 0 (AVBD, :64),
    // which it rejects, so CD stays as it was
    if (rows <= 0 || N <= 0 || a <= 0) return;
    const int a_eff = K > 0 ? (int)a : 0;  // an empty sum leaves AV^T BD = 0
    ThreadCtx &tc = thread_ctx();
    hcore_dense_task t{};
    t.kind = 3; t.M = rows; t.N = N; t.a = a_eff; t.kdim = std::max(K, 1);
    t.alpha = alpha; t.beta = beta;
    const bool dev = is_device_memory(CD) &&
                     (a_eff == 0 || (is_device_memory(AU) && is_device_memory(AV) &&
                                     is_device_memory(BD)));
    if (dev) {
        t.Au = AU; t.Av = AV; t.lda = LDA; t.Bd = BD; t.ldb = LDB; t.CD = CD; t.ldcd = LDC;
    } else {
        if (LDC < rows || (a_eff > 0 && (LDA < std::max(rows, K) || LDB < K)))
            fatal("HCORE_dgemmbdcd: invalid leading dimension (LDA %d, LDB %d, LDC %d)\n", LDA,
                  LDB, LDC);
        const int ld = std::max(rows, K);  // AU and AV share one leading dimension
        const size_t nf = (size_t)ld * a_eff, nd = (size_t)K * N;
        double *buf = stage_buffer(2 * nf + nd + (size_t)rows * N, "HCORE_dgemmbdcd");
        stage_ld(buf, ld, AU, rows, a_eff, LDA, tc.stream);
        stage_ld(buf + nf, ld, AV, K, a_eff, LDA, tc.stream);
        if (a_eff) stage(buf + 2 * nf, BD, K, N, LDB, tc.stream);
        stage(buf + 2 * nf + nd, CD, rows, N, LDC, tc.stream);
        t.Au = buf; t.Av = buf + nf; t.lda = ld; t.Bd = buf + 2 * nf; t.ldb = K;
        t.CD = buf + 2 * nf + nd; t.ldcd = rows;
    }
    if (run_dense(1, &t, tc.stream, true)) fatal("HCORE_dgemmbdcd: %s\n", last_error());
    if (!dev) unstage(CD, LDC, t.CD, rows, N, tc.stream, "HCORE_dgemmbdcd");
}

}  // extern "C"

template <typename T>
static void dense_gemm(const char *fn, int transA, int transB, int M, int N, int K, T alpha,
                       const T *A, int LDA, const T *B, int LDB, T beta, T *C, int LDC) {
    ThreadCtx &tc = thread_ctx();
    const int ta = transA == HCORE_Trans || transA == HCORE_ConjTrans;
    const int tb = transB == HCORE_Trans || transB == HCORE_ConjTrans;
    const int ar = ta ? K : M, ac = ta ? M : K, br = tb ? N : K, bc = tb ? K : N;
    const bool dev = is_device_memory(A) && is_device_memory(B) && is_device_memory(C);
    if (dev) {
        if (launch_gemm_dense<T>(ta, tb, M, N, K, alpha, A, LDA, B, LDB, beta, C, LDC, tc.stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(tc.stream) != cudaSuccess)
            cuda_fatal(fn);
        return;
    }
    const size_t na = (size_t)ar * ac, nb = (size_t)br * bc, nc = (size_t)M * N;
    T *buf = (T *)tc.dev_ensure((na + nb + nc) * sizeof(T) + 256);
    if (!buf) cuda_fatal(fn);
    T *dA = buf, *dB = buf + na, *dC = buf + na + nb;
    auto h2d = [&](T *dst, const T *src, int rows, int cols, int ld) {
        if (rows > 0 && cols > 0)
            cudaMemcpy2DAsync(dst, rows * sizeof(T), src, (size_t)ld * sizeof(T), rows * sizeof(T),
                              cols, cudaMemcpyHostToDevice, tc.stream);
    };
    h2d(dA, A, ar, ac, LDA);
    h2d(dB, B, br, bc, LDB);
    h2d(dC, C, M, N, LDC);
    if (launch_gemm_dense<T>(ta, tb, M, N, K, alpha, dA, ar, dB, br, beta, dC, M, tc.stream) !=
        cudaSuccess)
        cuda_fatal(fn);
    if (M > 0 && N > 0)
        cudaMemcpy2DAsync(C, (size_t)LDC * sizeof(T), dC, M * sizeof(T), M * sizeof(T), N,
                          cudaMemcpyDeviceToHost, tc.stream);
    if (cudaStreamSynchronize(tc.stream) != cudaSuccess) cuda_fatal(fn);
}

extern "C" {

void HCORE_dgemm_dense(HCORE_enum transA, int transB, int M, int N, int K, double alpha,
                       const double *A, int LDA, const double *B, int LDB, double beta,
                       double *C, int LDC) {
    dense_gemm<double>("HCORE_dgemm_dense", transA, transB, M, N, K, alpha, A, LDA, B, LDB, beta,
                       C, LDC);
}

void HCORE_sgemm_dense(HCORE_enum transA, int transB, int M, int N, int K, float alpha,
                       const float *A, int LDA, const float *B, int LDB, float beta, float *C,
                       int LDC) {
    dense_gemm<float>("HCORE_sgemm_dense", transA, transB, M, N, K, alpha, A, LDA, B, LDB, beta,
                      C, LDC);
}

static int translate_dense(int n, const hcore_dense_task *tasks, std::vector<hcore_dense_task> &tt) {
    tt.assign(tasks, tasks + n);
    for (auto &t : tt) {
        // only the pointers each kind reads (hcore_dense_task in hcore_gb300.h)
        const bool uses_av = t.kind != 2, uses_b = t.kind == 1, uses_bv = t.kind == 1 || t.kind == 2;
        const bool factors = t.kind <= 1 || t.a > 0;
        bool ok = true;
        auto tr = [&](const double *&p, bool used) {
            if (!used) return;
            p = (const double *)device_alias(p);
            ok = ok && p != nullptr;
        };
        tr(t.Au, factors);
        tr(t.Av, factors && uses_av);
        tr(t.Bu, uses_b);
        tr(t.Bv, factors && uses_bv);
        tr(t.Bd, t.kind == 3 && t.a > 0);
        t.CD = (double *)device_alias(t.CD);
        if (!ok || !t.CD) {
            set_error("hcore_gpu_dense_batched: pointers must be device or pinned memory");
            return HCORE_GPU_EINVAL;
        }
    }
    return HCORE_GPU_OK;
}

int hcore_gpu_dense_batched(int n, const hcore_dense_task *tasks, void *stream) {
    if (n < 0 || (n > 0 && !tasks)) {
        set_error("hcore_gpu_dense_batched: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    std::vector<hcore_dense_task> tt;
    int rc = translate_dense(n, tasks, tt);
    if (rc) return rc;
    return run_dense(n, tt.data(), (cudaStream_t)stream, true);
}

}  // extern "C"

struct hcore_gpu_dense_plan_s {
    DensePrep prep;
    char *arena = nullptr;
};

extern "C" {

int hcore_gpu_dense_plan_create(hcore_gpu_dense_plan *plan, int n, const hcore_dense_task *tasks) {
    if (!plan || n < 0 || (n > 0 && !tasks)) {
        set_error("hcore_gpu_dense_plan_create: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    *plan = nullptr;
    std::vector<hcore_dense_task> tt;
    int rc = translate_dense(n, tasks, tt);
    if (rc) return rc;
    auto *p = new hcore_gpu_dense_plan_s;
    rc = p->prep.build(n, tt.data());
    if (rc) {
        delete p;
        return rc;
    }
    if (cudaMalloc(&p->arena, std::max<size_t>(p->prep.bytes(), 256)) != cudaSuccess) {
        cudaGetLastError();
        set_error("hcore_gpu_dense_plan_create: cudaMalloc of %zu bytes failed", p->prep.bytes());
        delete p;
        return HCORE_GPU_ENOMEM;
    }
    p->prep.bind(tt.data(), (const double *)(p->arena + p->prep.ws_offset()));
    std::vector<char> host(p->prep.ws_offset());
    p->prep.pack(host.data(), tt.data());
    if (cudaMemcpy(p->arena, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("hcore_gpu_dense_plan_create: upload failed");
        cudaFree(p->arena);
        delete p;
        return HCORE_GPU_ECUDA;
    }
    *plan = p;
    return HCORE_GPU_OK;
}

int hcore_gpu_dense_plan_execute(hcore_gpu_dense_plan p, void *stream) {
    if (!p) {
        set_error("hcore_gpu_dense_plan_execute: null plan");
        return HCORE_GPU_EINVAL;
    }
    if (p->prep.n == 0) return HCORE_GPU_OK;
    const cudaError_t e = p->prep.launch(p->arena, (cudaStream_t)stream);
    if (e != cudaSuccess) {
        set_error("hcore_gpu_dense_plan_execute: %s", cudaGetErrorString(e));
        return HCORE_GPU_ECUDA;
    }
    return HCORE_GPU_OK;
}

int hcore_gpu_dense_plan_destroy(hcore_gpu_dense_plan p) {
    if (p) {
        cudaFree(p->arena);
        delete p;
    }
    return HCORE_GPU_OK;
}

void *hcore_gpu_thread_stream(void) { return (void *)thread_ctx().stream; }

}  // extern "C"

// ---- HCORE_zgemm through the real pipeline ----------------------------------
// A complex m x n matrix X embeds as the real 2m x 2n matrix
//     phi(X) = [Re X, -Im X; Im X, Re X],
// with phi(X Y^T) = phi(X) psi(Y)^T where psi(Y) = phi(conj Y).  So
//     phi(C) = phi(beta CU) psi(CV)^T,
//     phi(A B^T) = phi(alpha AU) psi(AV)^T (psi(BU) phi(BV)^T)^T,
// a real update of order 2M with ranks 2a, 2b, 2c, which the real plan
// recompresses (maxrk and rk doubled: phi(X) has each singular value of X
// twice, so the real rank rule keeps whole pairs).  The truncated real
// product is phi(C_new), whose left block column gives C_new = Z0 R^T with
// Z0 = CU'_top + i CU'_bottom and R = CV'_top.  The complex factors are an
// orthonormal basis Z of Z0's columns (modified Gram-Schmidt in column order,
// keeping a column when at least half of it is new: one column per pair of
// equal singular values) and CV = C_new^T conj(Z) = R (Z0^T conj(Z)), so
// CU CV^T = Z Z^H C_new = C_new.  In column order the basis vectors are
// C_new's left singular vectors and CV carries the singular values, as in
// the reference (hcore_zgemm.c:380-430).
namespace hc {
using zc = std::complex<double>;

// copy a complex block (rows x cols, ld) from host or device memory
static std::vector<zc> zget(const hcore_dcomplex *p, int rows, int cols, int ld) {
    std::vector<zc> out((size_t)rows * cols);
    if (rows > 0 && cols > 0 &&
        cudaMemcpy2D(out.data(), rows * sizeof(zc), p, (size_t)ld * sizeof(zc), rows * sizeof(zc),
                     cols, cudaMemcpyDefault) != cudaSuccess)
        cuda_fatal("HCORE_zgemm");
    return out;
}

// Complex factors of C_new from the real plan's outputs eU, eV (2M x r2,
// ld 2M): C_new = Z0 R^T, Z0 = eU_top + i eU_bottom, R = eV_top.  With
// `mgs` false, one column per pair is taken directly (column 2j; its
// partner must be J = [0 -I; I 0] times it, which is checked): CU_j =
// Z0_{2j}, CV_j = eV_top_{2j} - i eV_bottom_{2j}.  Where the check fails
// (singular values that are equal, so that pairs mix) or with `mgs` true,
// an orthonormal basis Z of Z0's columns is taken instead (modified
// Gram-Schmidt in column order, a column kept when more than half of it is
// new) and CV = R (Z0^T conj Z).  Returns the complex rank.
static int zextract(const double *eU, const double *eV, int M, int r2, bool mgs,
                    std::vector<zc> &oU, std::vector<zc> &oV) {
    const size_t M2 = 2 * (size_t)M;
    if (!mgs) {
        for (int j = 0; j + 1 < r2 && !mgs; j += 2) {  // partner == +-J * column
            const double *u = eU + (size_t)j * M2, *w = eU + (size_t)(j + 1) * M2;
            double d = 0;
            for (int i = 0; i < M; ++i) d += w[i] * -u[M + i] + w[M + i] * u[i];
            if (std::fabs(std::fabs(d) - 1.0) > 1e-6) mgs = true;
        }
    }
    if (!mgs) {
        const int r = (r2 + 1) / 2;
        oU.assign((size_t)M * r, zc());
        oV.assign((size_t)M * r, zc());
        for (int q = 0; q < r; ++q) {
            const double *u = eU + (size_t)(2 * q) * M2, *v = eV + (size_t)(2 * q) * M2;
            for (int i = 0; i < M; ++i) {
                oU[(size_t)q * M + i] = zc(u[i], u[M + i]);
                oV[(size_t)q * M + i] = zc(v[i], -v[M + i]);
            }
        }
        return r;
    }
    std::vector<zc> Z0((size_t)M * r2), Z;
    for (int j = 0; j < r2; ++j)
        for (int i = 0; i < M; ++i)
            Z0[(size_t)j * M + i] = zc(eU[(size_t)j * M2 + i], eU[(size_t)j * M2 + M + i]);
    int r = 0;
    std::vector<zc> z(M);
    for (int j = 0; j < r2; ++j) {
        double n0 = 0;
        for (int i = 0; i < M; ++i) {
            z[i] = Z0[(size_t)j * M + i];
            n0 += std::norm(z[i]);
        }
        for (int pass = 0; pass < 2; ++pass)
            for (int q = 0; q < r; ++q) {
                zc h = 0;
                for (int i = 0; i < M; ++i) h += std::conj(Z[(size_t)q * M + i]) * z[i];
                for (int i = 0; i < M; ++i) z[i] -= h * Z[(size_t)q * M + i];
            }
        double n1 = 0;
        for (int i = 0; i < M; ++i) n1 += std::norm(z[i]);
        if (n0 > 0 && n1 > 0.25 * n0) {
            const double inv = 1.0 / std::sqrt(n1);
            for (int i = 0; i < M; ++i) Z.push_back(z[i] * inv);
            ++r;
        }
    }
    std::vector<zc> G((size_t)r2 * r);
    for (int q = 0; q < r; ++q)
        for (int j = 0; j < r2; ++j) {
            zc g = 0;
            for (int i = 0; i < M; ++i) g += Z0[(size_t)j * M + i] * std::conj(Z[(size_t)q * M + i]);
            G[(size_t)q * r2 + j] = g;
        }
    oU.assign((size_t)M * r, zc());
    oV.assign((size_t)M * r, zc());
    for (int q = 0; q < r; ++q)
        for (int i = 0; i < M; ++i) {
            zc v = 0;
            for (int j = 0; j < r2; ++j) v += eV[(size_t)j * M2 + i] * G[(size_t)q * r2 + j];
            oV[(size_t)q * M + i] = v;
            oU[(size_t)q * M + i] = Z[(size_t)q * M + i];
        }
    return r;
}
}  // namespace hc

extern "C" void HCORE_zgemm(HCORE_enum transA, int transB, int M, int N, hcore_dcomplex alpha,
                            hcore_dcomplex *AU, hcore_dcomplex *AV, double *Ark, int LDA,
                            hcore_dcomplex *BU, hcore_dcomplex *BV, double *Brk, int LDB,
                            hcore_dcomplex beta, hcore_dcomplex *CU, hcore_dcomplex *CV,
                            double *Crk, int LDC, int rk, int maxrk, double acc,
                            hcore_dcomplex *work, flop_counter *flops) {
    (void)transA; (void)transB; (void)N; (void)work;
    const char *fn = "HCORE_zgemm";
    const int a = (int)Ark[0], b = (int)Brk[0], c = (int)Crk[0];
    // the reference's exits (hcore_zgemm.c:703-706 and __zqra/ld_newV as in
    // HCORE_dgemm), on the complex ranks
    if (a == 0 || b == 0 || c == 0)
        fatal("%s: _Ark=%d _Brk=%d _Crk=%d. These rank values should not be zero.\n", fn, a, b, c);
    if (a + c > 2 * maxrk)
        fatal("%s: Sum of ranks (%d) is too big! _Ark:%d _Crk:%d maxrank:%d (x2: %d)\n", fn,
              a + c, a, c, maxrk, 2 * maxrk);
    if (maxrk < a + c)
        fatal("%s: Increase maxrank. %d is not enough ld_newV:%d CU_ncols:%d\n", fn, maxrk,
              maxrk, a + c);
    if (2 * M > kMaxRowsPerLane * 32 || 2 * (a + c) > kMaxK)
        fatal("%s: M=%d, a+c=%d exceed this library's complex limits (M <= %d, a+c <= %d)\n", fn,
              M, a + c, kMaxRowsPerLane * 16, kMaxK / 2);
    // one task of the batched complex path: embedding, the real plan and the
    // pair extraction on the GPU, CU/CV written in place
    hcore_zlr_task t{};
    t.M = M; t.a = a; t.b = b; t.c = c; t.rk = rk; t.maxrk = maxrk;
    t.alpha = alpha; t.beta = beta; t.acc = acc;
    t.AU = AU; t.AV = AV; t.lda = LDA; t.BU = BU; t.BV = BV; t.ldb = LDB;
    t.CU = CU; t.CV = CV; t.ldc = LDC;
    int r = 0, st = 0;
    const int rc = hcore_gpu_zgemm_batched(1, &t, &r, &st, thread_ctx().stream);
    if (st == HCORE_GPU_S_RANK_MAX)  // hcore_zgemm.c's r > maxrk exit
        fatal("%s: Rank after truncation is too big! finalrank:%d maxrank:%d\n", fn, r, maxrk);
    if (rc == HCORE_GPU_ECUDA || rc == HCORE_GPU_ENOMEM) cuda_fatal(fn);
    if (rc != HCORE_GPU_OK || st != HCORE_GPU_S_OK)
        fatal("%s: recompression failed (status %d): %s\n", fn, st, last_error());
    Crk[0] = r;
    if (flops) flops->update += update_flops(M, a, b, c, r, false);  // hcore_zgemm.c: same model
}

// HCORE_zuncompress (src/compute/hcore_zuncompress.c:35-86): CD = AU BV^T
// in complex arithmetic (alpha and beta unused, Ark == Brk asserted), as two
// real uncompress tasks of rank 2a on the dense tile kernel:
//   Re CD = [Re AU, -Im AU] [Re BV, Im BV]^T,  Im CD = [Re AU, Im AU] [Im BV, Re BV]^T.
extern "C" void HCORE_zuncompress(HCORE_enum transA, HCORE_enum transB, int M, int N,
                                  hcore_dcomplex alpha, hcore_dcomplex *AU, double *Ark, int LDA,
                                  hcore_dcomplex *BV, double *Brk, int LDB, hcore_dcomplex beta,
                                  hcore_dcomplex *CD, int LDC) {
    (void)transA; (void)transB; (void)alpha; (void)beta;
    const char *fn = "HCORE_zuncompress";
    const long long a = (long long)Ark[0], b = (long long)Brk[0];
    if (a != b) fatal("%s: Ark (%lld) and Brk (%lld) must be equal\n", fn, a, b);
    if (M <= 0 || N <= 0) return;
    if (LDA < M || LDB < N || LDC < M)
        fatal("%s: invalid leading dimension (LDA %d, LDB %d, LDC %d)\n", fn, LDA, LDB, LDC);
    const int r = (int)a;
    const std::vector<zc> xU = zget(AU, M, r, LDA), xV = zget(BV, N, r, LDB);
    // host: [Re U | -Im U], [Re U | Im U] (M x 2r); [Re V | Im V], [Im V | Re V] (N x 2r)
    std::vector<double> h((size_t)2 * M * 2 * r + (size_t)2 * N * 2 * r);
    double *Pre = h.data(), *Pim = Pre + (size_t)M * 2 * r, *Qre = Pim + (size_t)M * 2 * r,
           *Qim = Qre + (size_t)N * 2 * r;
    for (int j = 0; j < r; ++j) {
        for (int i = 0; i < M; ++i) {
            const zc u = xU[(size_t)j * M + i];
            Pre[(size_t)j * M + i] = u.real(); Pre[(size_t)(r + j) * M + i] = -u.imag();
            Pim[(size_t)j * M + i] = u.real(); Pim[(size_t)(r + j) * M + i] = u.imag();
        }
        for (int i = 0; i < N; ++i) {
            const zc v = xV[(size_t)j * N + i];
            Qre[(size_t)j * N + i] = v.real(); Qre[(size_t)(r + j) * N + i] = v.imag();
            Qim[(size_t)j * N + i] = v.imag(); Qim[(size_t)(r + j) * N + i] = v.real();
        }
    }
    ThreadCtx &tc = thread_ctx();
    const size_t nin = h.size(), nout = (size_t)2 * M * N;
    double *buf = stage_buffer(nin + nout, fn);
    if (nin && cudaMemcpyAsync(buf, h.data(), nin * sizeof(double), cudaMemcpyHostToDevice,
                               tc.stream) != cudaSuccess)
        cuda_fatal(fn);
    double *dP = buf, *dQ = buf + (size_t)2 * M * 2 * r, *dOut = buf + nin;
    hcore_dense_task t[2] = {};
    for (int q = 0; q < 2; ++q) {
        t[q].kind = 2; t[q].M = M; t[q].N = N; t[q].a = 2 * r;
        t[q].Au = dP + (size_t)q * M * 2 * r; t[q].lda = M;
        t[q].Bv = dQ + (size_t)q * N * 2 * r; t[q].ldb = N;
        t[q].CD = dOut + (size_t)q * M * N; t[q].ldcd = M;
    }
    if (run_dense(2, t, tc.stream, true)) fatal("%s: %s\n", fn, last_error());
    std::vector<double> o(nout);
    if (cudaMemcpyAsync(o.data(), dOut, nout * sizeof(double), cudaMemcpyDeviceToHost,
                        tc.stream) != cudaSuccess ||
        cudaStreamSynchronize(tc.stream) != cudaSuccess)
        cuda_fatal(fn);
    std::vector<zc> z((size_t)M * N);
    for (size_t e = 0; e < (size_t)M * N; ++e) z[e] = zc(o[e], o[(size_t)M * N + e]);
    if (cudaMemcpy2D(CD, (size_t)LDC * sizeof(zc), z.data(), M * sizeof(zc), M * sizeof(zc), N,
                     cudaMemcpyDefault) != cudaSuccess)
        cuda_fatal(fn);
}

// run body(i) for i in [0, n) on up to 16 host threads
template <typename F>
static void parallel_for(int n, F body) {
    const int nt = std::max(1, std::min<int>({n, 16, (int)std::thread::hardware_concurrency()}));
    if (nt <= 1) {
        for (int i = 0; i < n; ++i) body(i);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([=, &body] {
            for (int i = t; i < n; i += nt) body(i);
        });
    for (auto &th : pool) th.join();
}

// Batched complex updates: every task embedded as above, all of them run as
// one real plan, the complex factors extracted per task (one column per pair
// of equal singular values, Gram-Schmidt where pairs mix).  The embedding
// and the pair extraction run on the GPU (zembed_kernel, zextract_kernel):
// only the complex factors cross the host link, and host inputs in pageable
// memory are packed on up to 16 threads into pinned memory that the kernel
// reads in place.
namespace hc {
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// one complex factor block (M x n, ld in complex elements, device-accessible)
// into its real embedding (2M x 2n, ld 2M), scaled by s, conjugated (psi) or
// not (phi)
struct ZEmbedBlock {
    const double *src;
    int ld;
    double *dst;
    int M, n;
    double sre, sim;
    int conj;
};
__global__ void __launch_bounds__(256) zembed_kernel(const ZEmbedBlock *__restrict__ blocks) {
    const ZEmbedBlock b = blocks[blockIdx.x];
    const size_t M = b.M, M2 = 2 * M, n = b.n;
    for (size_t e = threadIdx.x; e < M * n; e += blockDim.x) {
        const size_t i = e % M, j = e / M;
        const double xr = b.src[2 * (j * b.ld + i)], xi = b.src[2 * (j * b.ld + i) + 1];
        double re = b.sre * xr - b.sim * xi, im = b.sre * xi + b.sim * xr;
        if (b.conj) im = -im;
        b.dst[j * M2 + i] = re;
        b.dst[j * M2 + M + i] = im;
        b.dst[(n + j) * M2 + i] = -im;
        b.dst[(n + j) * M2 + M + i] = re;
    }
}
// the complex factors of one task from the real plan's outputs (eU, eV:
// 2M x r2, ld 2M): column 2q of each pair (CU_q = top + i bottom of eU,
// CV_q = top - i bottom of eV) into oU, oV (complex M x r, ld M); mixed = 1
// when some pair's partner is not +-J times its first column (singular
// values that are equal), which the host then resolves by Gram-Schmidt
struct ZExtractTask {
    const double *eU, *eV;
    int M, r2;
    double *oU, *oV;
};
__global__ void __launch_bounds__(256) zextract_kernel(const ZExtractTask *__restrict__ tasks,
                                                       int *__restrict__ mixed) {
    const ZExtractTask t = tasks[blockIdx.x];
    const size_t M = t.M, M2 = 2 * M;
    __shared__ double red[8];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    int mix = 0;
    for (int j = 0; j + 1 < t.r2; j += 2) {
        const double *u = t.eU + j * M2, *w = t.eU + (j + 1) * M2;
        double d = 0;
        for (size_t i = tid; i < M; i += blockDim.x) d += w[i] * -u[M + i] + w[M + i] * u[i];
        d = warp_sum_d(d);
        if (lane == 0) red[warp] = d;
        __syncthreads();
        if (tid == 0) {
            double s = 0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) s += red[q];
            if (fabs(fabs(s) - 1.0) > 1e-6) mix = 1;
        }
        __syncthreads();
    }
    if (tid == 0) mixed[blockIdx.x] = mix;
    const int r = (t.r2 + 1) / 2;
    for (size_t e = tid; e < M * (size_t)r; e += blockDim.x) {
        const size_t i = e % M, q = e / M;
        const double *u = t.eU + 2 * q * M2, *v = t.eV + 2 * q * M2;
        t.oU[2 * (q * M + i)] = u[i];
        t.oU[2 * (q * M + i) + 1] = u[M + i];
        t.oV[2 * (q * M + i)] = v[i];
        t.oV[2 * (q * M + i) + 1] = -v[M + i];
    }
}
}  // namespace hc

// Native complex path (hc_zkernels.cu): the tasks in `run` (validated) with
// M <= 1024 and a + c within the complex SVD's shared-memory limit.  Inputs
// in device memory are read in place; host inputs (pageable or pinned) are
// packed on the host into pinned staging and copied to the device in one
// transfer, because the stack kernel reads every factor column many times
// (F = AV^T BV, G = BU F^T), which over the host link would cost each read
// again.  The new factors are written to a device buffer and copied to the
// tasks' CU/CV.
static int zgemm_batched_native(const hcore_zlr_task *tasks, const std::vector<int> &run,
                                int *ranks, int *status, cudaStream_t s) {
    const int nr = (int)run.size();
    struct Src {
        const hcore_dcomplex *p;
        int rows, cols, ld;
    };
    std::vector<Src> src;
    std::vector<const zd *> where;     // device-accessible address, or null: packed
    std::vector<size_t> pack_off;
    std::vector<long long> ws_off(nr);
    std::vector<size_t> out_off(nr);
    size_t n_pack = 0, n_out = 0;
    long long n_ws = 0;
    int maxM = 1, maxK = 1;
    for (int x = 0; x < nr; ++x) {
        const hcore_zlr_task &t = tasks[run[x]];
        const Src f[6] = {{t.AU, t.M, t.a, t.lda}, {t.AV, t.M, t.a, t.lda},
                          {t.BU, t.M, t.b, t.ldb}, {t.BV, t.M, t.b, t.ldb},
                          {t.CU, t.M, t.c, t.ldc}, {t.CV, t.M, t.c, t.ldc}};
        for (const Src &b : f) {
            src.push_back(b);
            const bool dev = is_device_memory(b.p);
            where.push_back(dev ? (const zd *)b.p : nullptr);
            pack_off.push_back(dev ? SIZE_MAX : n_pack);
            if (!dev) n_pack += (size_t)b.rows * b.cols;
        }
        const int k = t.a + t.c;
        ws_off[x] = n_ws;
        n_ws += zlayout(t.M, t.a, t.b, k).total;
        out_off[x] = n_out;
        n_out += 2 * (size_t)t.M * k;
        maxM = std::max(maxM, t.M);
        maxK = std::max(maxK, k);
    }
    ThreadCtx &tc = thread_ctx();
    const size_t stage = std::max(n_pack, n_out) * sizeof(zd);
    zd *pin = (zd *)tc.pin_ensure(std::max<size_t>(stage, 1024));
    const size_t b_ws = al256((size_t)n_ws * sizeof(zd)), b_out = al256(n_out * sizeof(zd));
    const size_t b_in = al256(n_pack * sizeof(zd));
    const size_t b_desc = al256((size_t)nr * sizeof(ZDesc)), b_rs = al256(2 * (size_t)nr * sizeof(int));
    char *arena = nullptr;
    if (!pin || cudaMalloc(&arena, b_ws + b_out + b_in + b_desc + b_rs) != cudaSuccess) {
        cudaGetLastError();
        set_error("hcore_gpu_zgemm_batched: allocation of %zu bytes failed",
                  b_ws + b_out + b_in + b_desc + b_rs);
        return HCORE_GPU_ENOMEM;
    }
    zd *dws = (zd *)arena, *dout = (zd *)(arena + b_ws), *din = (zd *)(arena + b_ws + b_out);
    ZDesc *ddesc = (ZDesc *)(arena + b_ws + b_out + b_in);
    int *drank = (int *)(arena + b_ws + b_out + b_in + b_desc), *dstat = drank + nr;
    cudaStreamSynchronize(tc.stream);   // the staging may still feed an earlier copy
    parallel_for((int)src.size(), [&](int bi) {
        if (pack_off[bi] == SIZE_MAX) return;
        const Src &b = src[bi];
        zd *dst = pin + pack_off[bi];
        for (int j = 0; j < b.cols; ++j)
            std::memcpy(dst + (size_t)j * b.rows, b.p + (size_t)j * b.ld, sizeof(zd) * b.rows);
    });
    std::vector<ZDesc> desc(nr);
    for (int x = 0; x < nr; ++x) {
        const hcore_zlr_task &t = tasks[run[x]];
        const zd *pt[6];
        int ldv[6];
        for (int f = 0; f < 6; ++f) {
            const size_t bi = (size_t)x * 6 + f;
            pt[f] = pack_off[bi] == SIZE_MAX ? where[bi] : din + pack_off[bi];
            ldv[f] = pack_off[bi] == SIZE_MAX ? src[bi].ld : src[bi].rows;
        }
        ZDesc &d = desc[x];
        d = ZDesc{};
        d.AU = pt[0]; d.AV = pt[1]; d.BU = pt[2]; d.BV = pt[3]; d.CU = pt[4]; d.CV = pt[5];
        d.ldau = ldv[0]; d.ldav = ldv[1]; d.ldbu = ldv[2];
        d.ldbv = ldv[3]; d.ldcu = ldv[4]; d.ldcv = ldv[5];
        const int k = t.a + t.c;
        d.CUo = dout + out_off[x];
        d.CVo = d.CUo + (size_t)t.M * k;
        d.ldco = t.M;
        d.ws = ws_off[x];
        d.alpha = zd{t.alpha.re, t.alpha.im};
        d.beta = zd{t.beta.re, t.beta.im};
        d.acc = t.acc;
        d.M = t.M; d.a = t.a; d.b = t.b; d.c = t.c; d.k = k;
        d.rk = t.rk;
        d.max_rank = t.maxrk;
        d.idx = x;
        d.status0 = 0;
    }
    int rc = HCORE_GPU_OK;
    std::vector<int> rs(2 * nr);
    if ((n_pack > 0 &&
         cudaMemcpyAsync(din, pin, n_pack * sizeof(zd), cudaMemcpyHostToDevice, s) !=
             cudaSuccess) ||
        cudaMemcpyAsync(ddesc, desc.data(), nr * sizeof(ZDesc), cudaMemcpyHostToDevice, s) !=
            cudaSuccess ||
        launch_zrecompress(ddesc, nr, dws, drank, dstat, maxM, maxK, s) != cudaSuccess ||
        cudaMemcpyAsync(rs.data(), drank, 2 * nr * sizeof(int), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess ||
        cudaMemcpyAsync(pin, dout, n_out * sizeof(zd), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        set_error("hcore_gpu_zgemm_batched: %s", cudaGetErrorString(cudaGetLastError()));
        rc = HCORE_GPU_ECUDA;
    }
    cudaFree(arena);
    if (rc) return rc;
    std::vector<int> copy_failed(nr, 0);
    parallel_for(nr, [&](int x) {
        const hcore_zlr_task &t = tasks[run[x]];
        const int q = run[x], r = rs[x], st = rs[nr + x];
        status[q] = st;
        if (st) return;
        const int M = t.M, k = t.a + t.c;
        const zd *pU = pin + out_off[x], *pV = pU + (size_t)M * k;
        if (r > 0) {
            if (is_device_memory(t.CU) || is_device_memory(t.CV)) {
                if (cudaMemcpy2D(t.CU, (size_t)t.ldc * sizeof(zd), pU, M * sizeof(zd),
                                 M * sizeof(zd), r, cudaMemcpyDefault) != cudaSuccess ||
                    cudaMemcpy2D(t.CV, (size_t)t.ldc * sizeof(zd), pV, M * sizeof(zd),
                                 M * sizeof(zd), r, cudaMemcpyDefault) != cudaSuccess)
                    copy_failed[x] = 1;
            } else {
                for (int j = 0; j < r; ++j) {
                    std::memcpy(t.CU + (size_t)j * t.ldc, pU + (size_t)j * M, M * sizeof(zd));
                    std::memcpy(t.CV + (size_t)j * t.ldc, pV + (size_t)j * M, M * sizeof(zd));
                }
            }
        }
        ranks[q] = r;
    });
    for (int x = 0; x < nr; ++x)
        if (copy_failed[x]) {
            set_error("hcore_gpu_zgemm_batched: output copy failed");
            return HCORE_GPU_ECUDA;
        }
    return HCORE_GPU_OK;
}

extern "C" int hcore_gpu_zgemm_batched(int n, const hcore_zlr_task *tasks, int *ranks,
                                       int *status, void *stream) {
    if (n < 0 || (n > 0 && (!tasks || !ranks || !status))) {
        set_error("hcore_gpu_zgemm_batched: invalid argument");
        return HCORE_GPU_EINVAL;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // validation on the complex ranks (the reference's exit conditions)
    std::vector<int> run;
    std::vector<size_t> off_in, off_out, off_z;
    size_t n_in = 0, n_out = 0, n_z = 0;
    for (int q = 0; q < n; ++q) {
        const hcore_zlr_task &t = tasks[q];
        ranks[q] = 0;
        int st = HCORE_GPU_S_OK;
        if (t.a <= 0 || t.b <= 0 || t.c <= 0) st = HCORE_GPU_S_ZERO_RANK;
        else if (t.a + t.c > 2 * t.maxrk) st = HCORE_GPU_S_RANK_SUM;
        else if (t.maxrk < t.a + t.c) st = HCORE_GPU_S_LDNEWV;
        else if (t.M < 1 || 2 * t.M > kMaxRowsPerLane * 32 || 2 * (t.a + t.c) > kMaxK ||
                 t.a + t.c > t.M || t.lda < t.M || t.ldb < t.M || t.ldc < t.M)
            st = HCORE_GPU_S_SHAPE;
        status[q] = st;
        if (st) continue;
        run.push_back(q);
        const size_t M2 = 2 * (size_t)t.M;
        off_in.push_back(n_in);
        n_in += M2 * 2 * (2 * (size_t)t.a + 2 * (size_t)t.b + 2 * (size_t)t.c);
        off_out.push_back(n_out);
        n_out += 2 * M2 * 2 * (size_t)(t.a + t.c);
        off_z.push_back(n_z);
        n_z += 2 * 2 * (size_t)t.M * (size_t)(t.a + t.c);   // complex CU, CV (a + c columns)
    }
    const int nr = (int)run.size();
    if (nr == 0) return n ? HCORE_GPU_ETASK : HCORE_GPU_OK;

    // native complex kernels where every task fits them (M <= 1024, both
    // Jacobi matrices in shared memory); the real embedding otherwise
    {
        const int zk = zsvd_kmax();
        bool native = zk > 0 && !getenv("HCORE_GPU_ZGEMM_EMBED");
        for (int x = 0; x < nr && native; ++x) {
            const hcore_zlr_task &t = tasks[run[x]];
            native = t.M <= 1024 && t.a + t.c <= zk;
        }
        if (native) {
            const int rcn = zgemm_batched_native(tasks, run, ranks, status, s);
            if (rcn) return rcn;
            bool any = false;
            for (int q = 0; q < n && !any; ++q) any = status[q] != 0;
            return any ? HCORE_GPU_ETASK : HCORE_GPU_OK;
        }
    }

    // complex inputs the kernel cannot read in place (pageable host memory)
    // are packed into pinned staging; the rest are read where they are
    struct Src {
        const hcore_dcomplex *p;
        int rows, cols, ld;
    };
    std::vector<Src> src;
    std::vector<const double *> src_dev;   // device-accessible address per block
    std::vector<size_t> pack_off;          // offset in the staging (doubles), or SIZE_MAX
    size_t n_pack = 0;
    for (int x = 0; x < nr; ++x) {
        const hcore_zlr_task &t = tasks[run[x]];
        const Src f[6] = {{t.AU, t.M, t.a, t.lda}, {t.AV, t.M, t.a, t.lda},
                          {t.BU, t.M, t.b, t.ldb}, {t.BV, t.M, t.b, t.ldb},
                          {t.CU, t.M, t.c, t.ldc}, {t.CV, t.M, t.c, t.ldc}};
        for (const Src &b : f) {
            src.push_back(b);
            const void *alias = device_alias(b.p);
            src_dev.push_back((const double *)alias);
            if (alias) {
                pack_off.push_back(SIZE_MAX);
            } else {
                pack_off.push_back(n_pack);
                n_pack += 2 * (size_t)b.rows * b.cols;
            }
        }
    }
    ThreadCtx &tc = thread_ctx();
    const size_t n_blocks = src.size();
    const size_t stage_doubles = std::max(n_pack, n_z);
    double *pin = (double *)tc.pin_ensure(std::max<size_t>(stage_doubles * sizeof(double), 1024));
    const size_t b_in = al256(n_in * sizeof(double)), b_out = al256(n_out * sizeof(double));
    const size_t b_z = al256(n_z * sizeof(double));
    const size_t b_blk = al256(n_blocks * sizeof(ZEmbedBlock));
    const size_t b_ex = al256((size_t)nr * sizeof(ZExtractTask)), b_mix = al256(nr * sizeof(int));
    char *arena = nullptr;
    if (!pin || cudaMalloc(&arena, b_in + b_out + b_z + b_blk + b_ex + b_mix) != cudaSuccess) {
        cudaGetLastError();
        set_error("hcore_gpu_zgemm_batched: allocation of %zu bytes failed",
                  b_in + b_out + b_z + b_blk + b_ex + b_mix);
        return HCORE_GPU_ENOMEM;
    }
    double *din = (double *)arena, *dout = (double *)(arena + b_in);
    double *dz = (double *)(arena + b_in + b_out);
    ZEmbedBlock *dblk = (ZEmbedBlock *)(arena + b_in + b_out + b_z);
    ZExtractTask *dex = (ZExtractTask *)(arena + b_in + b_out + b_z + b_blk);
    int *dmix = (int *)(arena + b_in + b_out + b_z + b_blk + b_ex);
    // the pinned staging may have been used by an earlier call's copies
    cudaStreamSynchronize(tc.stream);
    parallel_for((int)n_blocks, [&](int bi) {
        if (pack_off[bi] == SIZE_MAX) return;
        const Src &b = src[bi];
        double *dst = pin + pack_off[bi];
        for (int j = 0; j < b.cols; ++j)
            std::memcpy(dst + 2 * (size_t)j * b.rows, b.p + (size_t)j * b.ld,
                        2 * sizeof(double) * b.rows);
    });
    const double *pin_dev = (const double *)device_alias(pin);
    std::vector<ZEmbedBlock> blk(n_blocks);
    std::vector<hcore_lr_task> rt(nr);
    for (int x = 0; x < nr; ++x) {
        const hcore_zlr_task &t = tasks[run[x]];
        const int M = t.M, a = t.a, b = t.b, c = t.c, M2 = 2 * M;
        double *e0 = din + off_in[x];
        double *eAU = e0, *eAV = eAU + (size_t)M2 * 2 * a, *eBU = eAV + (size_t)M2 * 2 * a,
               *eBV = eBU + (size_t)M2 * 2 * b, *eCU = eBV + (size_t)M2 * 2 * b,
               *eCV = eCU + (size_t)M2 * 2 * c;
        double *dst[6] = {eAU, eAV, eBU, eBV, eCU, eCV};
        const double sc[6][2] = {{t.alpha.re, t.alpha.im}, {1, 0}, {1, 0},
                                 {1, 0}, {t.beta.re, t.beta.im}, {1, 0}};
        const int cj[6] = {0, 1, 1, 0, 0, 1};   // phi(alpha AU) psi(AV), psi(BU) phi(BV), ...
        for (int f = 0; f < 6; ++f) {
            const size_t bi = (size_t)x * 6 + f;
            const Src &sb = src[bi];
            ZEmbedBlock &z = blk[bi];
            if (pack_off[bi] == SIZE_MAX) {
                z.src = src_dev[bi];
                z.ld = sb.ld;
            } else {
                z.src = pin_dev + pack_off[bi];
                z.ld = sb.rows;
            }
            z.dst = dst[f];
            z.M = M;
            z.n = sb.cols;
            z.sre = sc[f][0];
            z.sim = sc[f][1];
            z.conj = cj[f];
        }
        double *o = dout + off_out[x];
        hcore_lr_task &u = rt[x];
        u = hcore_lr_task{};
        u.M = M2; u.a = 2 * a; u.b = 2 * b; u.c = 2 * c; u.rk = 2 * t.rk; u.maxrk = 2 * t.maxrk;
        u.ld_newv = 2 * t.maxrk; u.alpha = 1.0; u.beta = 1.0; u.acc = t.acc;
        u.AU = eAU; u.AV = eAV; u.lda = M2;
        u.BU = eBU; u.BV = eBV; u.ldb = M2;
        u.CU = eCU; u.CV = eCV; u.ldc = M2;
        u.CUo = o; u.CVo = o + (size_t)M2 * 2 * (a + c); u.ldco = M2;
    }
    int rc = HCORE_GPU_OK;
    hcore_gpu_plan plan = nullptr;
    std::vector<int> r2(nr), st2(nr), mixed(nr, 0);
    if (cudaMemcpyAsync(dblk, blk.data(), n_blocks * sizeof(ZEmbedBlock), cudaMemcpyHostToDevice,
                        s) != cudaSuccess) {
        set_error("hcore_gpu_zgemm_batched: upload failed");
        rc = HCORE_GPU_ECUDA;
    }
    if (rc == HCORE_GPU_OK) {
        zembed_kernel<<<(unsigned)n_blocks, 256, 0, s>>>(dblk);
        if (cudaGetLastError() != cudaSuccess) {
            set_error("hcore_gpu_zgemm_batched: embedding kernel failed to launch");
            rc = HCORE_GPU_ECUDA;
        }
    }
    if (rc == HCORE_GPU_OK) rc = hcore_gpu_plan_create(&plan, HCORE_GPU_F64, nr, rt.data(), 0);
    if (rc == HCORE_GPU_OK) rc = hcore_gpu_plan_execute(plan, stream);
    if (rc == HCORE_GPU_OK) rc = hcore_gpu_plan_results(plan, r2.data(), st2.data(), stream);
    if (plan) hcore_gpu_plan_destroy(plan);
    if (rc == HCORE_GPU_OK) {
        std::vector<ZExtractTask> ex(nr);
        for (int x = 0; x < nr; ++x) {
            const hcore_zlr_task &t = tasks[run[x]];
            const int M2 = 2 * t.M;
            const double *eU = dout + off_out[x];
            ex[x] = ZExtractTask{eU, eU + (size_t)M2 * 2 * (t.a + t.c), t.M,
                                 st2[x] == HCORE_GPU_S_OK ? r2[x] : 0, dz + off_z[x],
                                 dz + off_z[x] + 2 * (size_t)t.M * (t.a + t.c)};
        }
        if (cudaMemcpyAsync(dex, ex.data(), nr * sizeof(ZExtractTask), cudaMemcpyHostToDevice,
                            s) != cudaSuccess) {
            rc = HCORE_GPU_ECUDA;
        } else {
            zextract_kernel<<<nr, 256, 0, s>>>(dex, dmix);
            if (cudaGetLastError() != cudaSuccess) rc = HCORE_GPU_ECUDA;
        }
        // the complex factors and the mixed flags back to the host (pinned)
        if (rc == HCORE_GPU_OK &&
            (cudaMemcpyAsync(pin, dz, n_z * sizeof(double), cudaMemcpyDeviceToHost, s) !=
                 cudaSuccess ||
             cudaMemcpyAsync(mixed.data(), dmix, nr * sizeof(int), cudaMemcpyDeviceToHost, s) !=
                 cudaSuccess ||
             cudaStreamSynchronize(s) != cudaSuccess))
            rc = HCORE_GPU_ECUDA;
        if (rc == HCORE_GPU_ECUDA) set_error("hcore_gpu_zgemm_batched: extraction failed");
    }
    // tasks whose pairs mixed: their real factors to the host for Gram-Schmidt
    std::vector<int> need;
    for (int x = 0; x < nr && rc == HCORE_GPU_OK; ++x)
        if (st2[x] == HCORE_GPU_S_OK && mixed[x]) need.push_back(x);
    std::vector<std::vector<double>> eh(need.size());
    for (size_t m = 0; m < need.size() && rc == HCORE_GPU_OK; ++m) {
        const int x = need[m];
        const hcore_zlr_task &t = tasks[run[x]];
        const size_t cnt = 2 * (2 * (size_t)t.M) * 2 * (t.a + t.c);
        eh[m].resize(cnt);
        if (cudaMemcpy(eh[m].data(), dout + off_out[x], cnt * sizeof(double),
                       cudaMemcpyDeviceToHost) != cudaSuccess) {
            set_error("hcore_gpu_zgemm_batched: download failed");
            rc = HCORE_GPU_ECUDA;
        }
    }
    cudaFree(arena);
    if (rc) return rc;
    std::vector<int> slot(nr, -1);
    for (size_t m = 0; m < need.size(); ++m) slot[need[m]] = (int)m;
    std::vector<int> copy_failed(nr, 0);
    parallel_for(nr, [&](int x) {
        const hcore_zlr_task &t = tasks[run[x]];
        const int q = run[x];
        status[q] = st2[x];
        if (st2[x]) return;
        const int M = t.M, M2 = 2 * M;
        std::vector<zc> oU, oV;
        const zc *pU, *pV;
        int r;
        if (slot[x] >= 0) {
            const double *eU = eh[slot[x]].data();
            r = zextract(eU, eU + (size_t)M2 * 2 * (t.a + t.c), M, r2[x], true, oU, oV);
            pU = oU.data();
            pV = oV.data();
        } else {
            r = (r2[x] + 1) / 2;
            pU = (const zc *)(pin + off_z[x]);
            pV = pU + (size_t)M * (t.a + t.c);
        }
        if (r > t.maxrk) {
            status[q] = HCORE_GPU_S_RANK_MAX;
            return;
        }
        if (r > 0) {
            if (is_device_memory(t.CU) || is_device_memory(t.CV)) {
                if (cudaMemcpy2D(t.CU, (size_t)t.ldc * sizeof(zc), pU, M * sizeof(zc),
                                 M * sizeof(zc), r, cudaMemcpyDefault) != cudaSuccess ||
                    cudaMemcpy2D(t.CV, (size_t)t.ldc * sizeof(zc), pV, M * sizeof(zc),
                                 M * sizeof(zc), r, cudaMemcpyDefault) != cudaSuccess)
                    copy_failed[x] = 1;
            } else {
                for (int j = 0; j < r; ++j) {
                    std::memcpy(t.CU + (size_t)j * t.ldc, pU + (size_t)j * M, M * sizeof(zc));
                    std::memcpy(t.CV + (size_t)j * t.ldc, pV + (size_t)j * M, M * sizeof(zc));
                }
            }
        }
        ranks[q] = r;
    });
    for (int x = 0; x < nr; ++x)
        if (copy_failed[x]) {
            set_error("hcore_gpu_zgemm_batched: output copy failed");
            return HCORE_GPU_ECUDA;
        }
    bool any = false;
    for (int q = 0; q < n && !any; ++q) any = status[q] != 0;
    return any ? HCORE_GPU_ETASK : HCORE_GPU_OK;
}
