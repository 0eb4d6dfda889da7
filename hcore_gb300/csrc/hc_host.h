// hcore-gb300 — host-side helpers shared by the plan API and the drop-in
// HCORE_* entry points.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "hc_internal.h"

namespace hc {

void set_error(const char *fmt, ...);
const char *last_error();
const void *device_alias(const void *p);
bool is_device_memory(const void *p);
int fill_desc(const hcore_lr_task &t, unsigned flags, bool translate, Desc &d, int &k_out);
void fill_buckets(const std::vector<Desc> &descs, LaunchShape &shape);
bool build_descs(int n, const hcore_lr_task *tasks, unsigned flags, bool translate,
                 std::vector<Desc> &descs, long long &ws_elems, int &maxM, int &maxK,
                 std::vector<int> *status0);

// Per-thread execution context of the drop-in entry points: a non-blocking
// stream, a growable device arena and a growable pinned staging buffer.  The
// reference is reentrant (every call mallocs its own buffers), so HiCMA calls
// it from many runtime worker threads at once; one context per thread keeps
// those calls independent.
struct ThreadCtx {
    cudaStream_t stream = nullptr;
    void *dev = nullptr;
    size_t dev_bytes = 0;
    void *pin = nullptr;
    size_t pin_bytes = 0;
    ~ThreadCtx();
    cudaError_t init();
    void *dev_ensure(size_t bytes);
    void *pin_ensure(size_t bytes);
};
ThreadCtx &thread_ctx();

// reference flop model of one update (src/misc/descutil/flop_counts.c:3-70
// as accumulated by hcore_dgemm.c:125,179,208,224,434,493,595,666)
unsigned long flop_counts(char op, unsigned long a, unsigned long b, unsigned long c,
                          unsigned long d);
unsigned long update_flops(int M, int a, int b, int c, int r, bool dense_b);

[[noreturn]] void fatal(const char *fmt, ...);

}  // namespace hc
